// wgsl.cpp — WGSL parser and CUDA emitter (see wgsl.h for the subset and its arithmetic).
#include "wgsl.h"

#include <algorithm>
#include <cctype>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <functional>
#include <map>
#include <set>
#include <sstream>
#include <tuple>

namespace gbr {
namespace wgsl {

[[noreturn]] static void bad(int line, const std::string& msg) {
    throw Error("WGSL line " + std::to_string(line) + ": " + msg, false);
}
[[noreturn]] static void unsupported(int line, const std::string& msg) {
    throw Error("WGSL line " + std::to_string(line) + ": unsupported: " + msg, true);
}

// ------------------------------------------------------------------------------------ lexer
enum class Tk { End, Ident, Int, Float, Punct };
struct Tok {
    Tk t = Tk::End;
    std::string s;
    int line = 0;
};

static std::vector<Tok> lex(const std::string& src) {
    static const char* puncts[] = {"<<=", ">>=", "->", "&&", "||", "==", "!=", "<=", ">=", "+=", "-=", "*=", "/=",
                                   "%=",  "&=",  "|=", "^=", "++", "--", "<<", ">>", "(",  ")",  "{",  "}",  "[",
                                   "]",   ",",   ";",  ":",  ".",  "@",  "=",  "<",  ">",  "+",  "-",  "*",  "/",
                                   "%",   "&",   "|",  "^",  "!",  "~"};
    std::vector<Tok> out;
    size_t i = 0;
    int line = 1;
    const size_t n = src.size();
    while (i < n) {
        char c = src[i];
        if (c == '\n') {
            ++line;
            ++i;
            continue;
        }
        if (std::isspace((unsigned char)c)) {
            ++i;
            continue;
        }
        if (c == '/' && i + 1 < n && src[i + 1] == '/') {
            while (i < n && src[i] != '\n') ++i;
            continue;
        }
        if (c == '/' && i + 1 < n && src[i + 1] == '*') {
            int depth = 0;
            do {
                if (src.compare(i, 2, "/*") == 0) {
                    ++depth;
                    i += 2;
                } else if (src.compare(i, 2, "*/") == 0) {
                    --depth;
                    i += 2;
                } else {
                    if (src[i] == '\n') ++line;
                    ++i;
                }
            } while (depth > 0 && i < n);
            continue;
        }
        Tok t;
        t.line = line;
        if (std::isalpha((unsigned char)c) || c == '_') {
            size_t j = i;
            while (j < n && (std::isalnum((unsigned char)src[j]) || src[j] == '_')) ++j;
            t.t = Tk::Ident;
            t.s = src.substr(i, j - i);
            i = j;
        } else if (std::isdigit((unsigned char)c) || (c == '.' && i + 1 < n && std::isdigit((unsigned char)src[i + 1]))) {
            size_t j = i;
            bool is_float = false;
            if (c == '0' && j + 1 < n && (src[j + 1] == 'x' || src[j + 1] == 'X')) {
                j += 2;
                while (j < n && std::isxdigit((unsigned char)src[j])) ++j;
            } else {
                while (j < n && std::isdigit((unsigned char)src[j])) ++j;
                if (j < n && src[j] == '.') {
                    is_float = true;
                    ++j;
                    while (j < n && std::isdigit((unsigned char)src[j])) ++j;
                }
                if (j < n && (src[j] == 'e' || src[j] == 'E')) {
                    is_float = true;
                    ++j;
                    if (j < n && (src[j] == '+' || src[j] == '-')) ++j;
                    while (j < n && std::isdigit((unsigned char)src[j])) ++j;
                }
            }
            if (j < n && (src[j] == 'f' || src[j] == 'h')) {
                is_float = true;
                ++j;
            } else if (j < n && (src[j] == 'i' || src[j] == 'u')) {
                ++j;
            }
            t.t = is_float ? Tk::Float : Tk::Int;
            t.s = src.substr(i, j - i);
            i = j;
        } else {
            bool found = false;
            for (const char* p : puncts) {
                size_t len = std::strlen(p);
                if (src.compare(i, len, p) == 0) {
                    t.t = Tk::Punct;
                    t.s = p;
                    i += len;
                    found = true;
                    break;
                }
            }
            if (!found) bad(line, std::string("unexpected character '") + c + "'");
        }
        out.push_back(t);
    }
    Tok e;
    e.line = line;
    out.push_back(e);
    return out;
}

// ------------------------------------------------------------------------------------ AST
struct TypeExpr {
    std::string name;
    std::vector<TypeExpr> args;
    std::string count;  // array length literal / constant name
    int line = 0;
};

struct Attr {
    std::string name;
    std::vector<std::string> args;
};

struct Expr;
using ExprP = std::shared_ptr<Expr>;
struct Expr {
    enum K { Lit, Ident, Member, Index, Call, Unary, Binary } k;
    std::string s;          // literal text, identifier, member, operator, callee
    TypeExpr callee_type;   // templated constructor (vec4<f32>(...), array<f32, 3>(...))
    bool templated = false;
    bool float_lit = false;
    std::vector<ExprP> a;
    int line = 0;
};

struct Stmt;
using StmtP = std::shared_ptr<Stmt>;
struct Stmt {
    enum K { Let, Var, Const, Assign, Incr, Decr, If, For, Loop, While, Break, BreakIf, Continue, Return, Discard,
             Switch, Block, Call } k;
    std::string name, op;
    bool has_type = false;
    TypeExpr ty;
    ExprP e, lhs;                    // value / condition / lvalue
    std::vector<StmtP> body, other;  // then / else, loop body / continuing
    StmtP init, update;              // for
    struct Case {
        std::vector<ExprP> values;
        bool is_default = false;
        std::vector<StmtP> body;
    };
    std::vector<Case> cases;
    int line = 0;
};

struct Member {
    std::string name;
    TypeExpr ty;
    std::vector<Attr> attrs;
};
struct StructDef {
    std::string name;
    std::vector<Member> members;
};
struct Global {
    enum K { Const, Private, Uniform, Texture, Sampler } k;
    std::string name;
    TypeExpr ty;
    bool has_type = false;
    ExprP init;
    int group = -1, binding = -1;
    int line = 0;
    bool is_override = false;     // `override`: a Const whose value the pipeline may set
    long long override_id = -1;   // its @id, or -1 (then the name is its key)
};
struct Func {
    std::string name;
    std::vector<Member> params;
    bool has_ret = false;
    TypeExpr ret;
    std::vector<Attr> ret_attrs;
    std::vector<Attr> attrs;  // the function's own attributes (@vertex, @early_depth_test, ...)
    std::vector<StmtP> body;
    int stage = -1;  // 0 vertex, 1 fragment, -1 helper
    int line = 0;
};

struct Module {
    std::vector<StructDef> structs;
    std::vector<Global> globals;
    std::vector<Func> funcs;
};

// ------------------------------------------------------------------------------------ parser
class Parser {
  public:
    explicit Parser(std::vector<Tok> toks) : t_(std::move(toks)) {}

    std::shared_ptr<Module> module() {
        auto m = std::make_shared<Module>();
        while (!at_end()) {
            std::vector<Attr> attrs = attributes();
            const int decl_line = line();
            auto no_attrs = [&](const char* what) {
                if (!attrs.empty()) bad(decl_line, "@" + attrs[0].name + " does not apply to " + what);
            };
            if (accept_kw("struct")) {
                no_attrs("a struct");
                m->structs.push_back(struct_def());
            } else if (accept_kw("fn")) {
                m->funcs.push_back(func(attrs));
            } else if (accept_kw("override")) {
                m->globals.push_back(override_decl(attrs));
                expect(";");
            } else if (peek_kw("const")) {
                no_attrs("a const");
                next();
                m->globals.push_back(global_value(Global::Const));
                expect(";");
            } else if (accept_kw("var")) {
                Global g;
                g.k = Global::Private;
                g.line = line();
                if (accept("<")) {
                    std::string space = ident();
                    if (space == "uniform") g.k = Global::Uniform;
                    else if (space == "private") g.k = Global::Private;
                    else unsupported(line(), "address space " + space);
                    expect(">");
                }
                g.name = ident();
                if (accept(":")) {
                    g.ty = type();
                    g.has_type = true;
                }
                if (accept("=")) g.init = expr();
                expect(";");
                if (g.has_type && g.ty.name == "texture_2d") g.k = Global::Texture;
                if (g.has_type && g.ty.name == "sampler") g.k = Global::Sampler;
                for (const Attr& a : attrs) {
                    if (a.name == "group" && !a.args.empty()) g.group = std::atoi(a.args[0].c_str());
                    else if (a.name == "binding" && !a.args.empty()) g.binding = std::atoi(a.args[0].c_str());
                    else bad(g.line, "@" + a.name + " does not apply to a module-scope var");
                }
                if (g.k != Global::Private && g.k != Global::Const && (g.group < 0 || g.binding < 0))
                    bad(g.line, "resource variable '" + g.name + "' needs @group and @binding");
                if (g.k != Global::Private && g.k != Global::Const && (g.group >= 4 || g.binding >= 8))
                    unsupported(g.line, "@group(" + std::to_string(g.group) + ") @binding(" + std::to_string(g.binding) +
                                            ") beyond 4 groups x 8 bindings");
                m->globals.push_back(g);
            } else if (accept_kw("alias")) {
                unsupported(line(), "type aliases");
            } else if (accept(";")) {
            } else if (peek_kw("enable") || peek_kw("requires") || peek_kw("diagnostic")) {
                unsupported(line(), "directive " + cur().s);
            } else {
                bad(line(), "unexpected '" + cur().s + "' at module scope");
            }
        }
        return m;
    }

  private:
    std::vector<Tok> t_;
    size_t p_ = 0;

    const Tok& cur() const { return t_[p_]; }
    int line() const { return t_[p_].line; }
    bool at_end() const { return t_[p_].t == Tk::End; }
    void next() {
        if (!at_end()) ++p_;
    }
    bool peek(const char* s) const { return t_[p_].t == Tk::Punct && t_[p_].s == s; }
    bool peek_kw(const char* s) const { return t_[p_].t == Tk::Ident && t_[p_].s == s; }
    bool accept(const char* s) {
        if (peek(s)) {
            next();
            return true;
        }
        // a `>>` closing two template lists
        if (std::strcmp(s, ">") == 0 && t_[p_].t == Tk::Punct && t_[p_].s == ">>") {
            t_[p_].s = ">";
            return true;
        }
        return false;
    }
    bool accept_kw(const char* s) {
        if (peek_kw(s)) {
            next();
            return true;
        }
        return false;
    }
    void expect(const char* s) {
        if (!accept(s)) bad(line(), std::string("expected '") + s + "', found '" + cur().s + "'");
    }
    std::string ident() {
        if (cur().t != Tk::Ident) bad(line(), "expected an identifier, found '" + cur().s + "'");
        std::string s = cur().s;
        next();
        return s;
    }

    // Attributes this front end acts on, and those with no effect on what is rendered (invariant:
    // the arithmetic here is deterministic anyway; must_use and diagnostic: checks and messages
    // only).  Everything else fails the module instead of being ignored.
    static void check_attribute(const std::string& n, int line) {
        static const char* const kUsed[] = {"location", "builtin", "interpolate", "group", "binding", "vertex",
                                            "fragment", "compute", "early_depth_test", "id", "invariant", "must_use",
                                            "diagnostic"};
        for (const char* k : kUsed)
            if (n == k) return;
        if (n == "align" || n == "size" || n == "blend_src" || n == "workgroup_size")
            unsupported(line, "attribute @" + n);
        bad(line, "unknown attribute @" + n);
    }

    std::vector<Attr> attributes() {
        std::vector<Attr> out;
        while (accept("@")) {
            Attr a;
            const int at_line = line();
            a.name = ident();
            check_attribute(a.name, at_line);
            if (accept("(")) {
                while (!peek(")")) {
                    if (cur().t == Tk::End) bad(line(), "unterminated attribute");
                    std::string v;
                    int depth = 0;
                    while (!(depth == 0 && (peek(",") || peek(")")))) {
                        if (peek("(")) ++depth;
                        if (peek(")")) --depth;
                        v += cur().s;
                        next();
                    }
                    a.args.push_back(v);
                    if (!accept(",")) break;
                }
                expect(")");
            }
            out.push_back(a);
        }
        return out;
    }

    TypeExpr type() {
        TypeExpr t;
        t.line = line();
        t.name = ident();
        if (accept("<")) {
            if (t.name == "array") {
                t.args.push_back(type());
                if (accept(",")) {
                    t.count = cur().s;
                    next();
                }
            } else if (t.name == "ptr") {
                unsupported(t.line, "pointer types");
            } else {
                t.args.push_back(type());
                while (accept(",")) t.args.push_back(type());
            }
            expect(">");
        }
        return t;
    }

    StructDef struct_def() {
        StructDef s;
        s.name = ident();
        expect("{");
        while (!accept("}")) {
            Member m;
            m.attrs = attributes();
            m.name = ident();
            expect(":");
            m.ty = type();
            s.members.push_back(m);
            if (!accept(",")) {
                expect("}");
                break;
            }
        }
        accept(";");
        return s;
    }

    // `override name [: type] [= initializer]` with an optional @id(n) (a pipeline-overridable
    // constant, set through PipelineCompilationOptions::constants)
    Global override_decl(const std::vector<Attr>& attrs) {
        Global g;
        g.k = Global::Const;
        g.is_override = true;
        g.line = line();
        g.name = ident();
        for (const Attr& a : attrs) {
            if (a.name != "id") bad(g.line, "@" + a.name + " does not apply to an override");
            if (a.args.size() != 1) bad(g.line, "@id takes one argument");
            char* end = nullptr;
            const long long id = std::strtoll(a.args[0].c_str(), &end, 0);
            if (!end || (*end && std::strcmp(end, "u") && std::strcmp(end, "i")) || id < 0 || id > 65535)
                bad(g.line, "@id must be an integer in [0, 65535]");
            g.override_id = id;
        }
        if (accept(":")) {
            g.ty = type();
            g.has_type = true;
        }
        if (accept("=")) g.init = expr();
        if (!g.has_type && !g.init) bad(g.line, "override '" + g.name + "' needs a type or an initializer");
        return g;
    }

    Global global_value(Global::K k) {
        Global g;
        g.k = k;
        g.line = line();
        g.name = ident();
        if (accept(":")) {
            g.ty = type();
            g.has_type = true;
        }
        expect("=");
        g.init = expr();
        return g;
    }

    Func func(const std::vector<Attr>& attrs) {
        Func f;
        f.line = line();
        f.name = ident();
        f.attrs = attrs;
        for (const Attr& a : attrs) {
            if (a.name == "vertex") f.stage = 0;
            else if (a.name == "fragment") f.stage = 1;
            else if (a.name == "compute") unsupported(f.line, "compute entry points");
            else if (a.name != "early_depth_test" && a.name != "must_use" && a.name != "diagnostic")
                bad(f.line, "@" + a.name + " does not apply to a function");
        }
        for (const Attr& a : attrs)
            if (a.name == "early_depth_test" && f.stage != 1) bad(f.line, "@early_depth_test applies to fragment entry points");
        expect("(");
        while (!accept(")")) {
            Member p;
            p.attrs = attributes();
            p.name = ident();
            expect(":");
            p.ty = type();
            f.params.push_back(p);
            if (!accept(",")) {
                expect(")");
                break;
            }
        }
        if (accept("->")) {
            f.ret_attrs = attributes();
            f.ret = type();
            f.has_ret = true;
        }
        f.body = block();
        return f;
    }

    std::vector<StmtP> block() {
        expect("{");
        std::vector<StmtP> out;
        while (!accept("}")) {
            if (at_end()) bad(line(), "unterminated block");
            StmtP s = statement();
            if (s) out.push_back(s);
        }
        return out;
    }

    StmtP mk(Stmt::K k) {
        auto s = std::make_shared<Stmt>();
        s->k = k;
        s->line = line();
        return s;
    }

    // a statement that can appear in for-init / for-update / plain position (no trailing ';')
    StmtP simple_statement() {
        if (peek_kw("let") || peek_kw("var") || peek_kw("const")) {
            std::string kw = cur().s;
            StmtP s = mk(kw == "let" ? Stmt::Let : kw == "var" ? Stmt::Var : Stmt::Const);
            next();
            if (kw == "var" && accept("<")) unsupported(s->line, "address space on a function variable");
            s->name = ident();
            if (accept(":")) {
                s->ty = type();
                s->has_type = true;
            }
            if (accept("=")) s->e = expr();
            else if (kw != "var") bad(s->line, kw + " '" + s->name + "' needs an initializer");
            return s;
        }
        if (peek_kw("_") ) {
            StmtP s = mk(Stmt::Call);
            next();
            expect("=");
            s->e = expr();
            return s;
        }
        ExprP lhs = expr();
        if (accept("++")) {
            StmtP s = mk(Stmt::Incr);
            s->lhs = lhs;
            return s;
        }
        if (accept("--")) {
            StmtP s = mk(Stmt::Decr);
            s->lhs = lhs;
            return s;
        }
        static const char* ops[] = {"=", "+=", "-=", "*=", "/=", "%=", "&=", "|=", "^=", "<<=", ">>="};
        for (const char* op : ops) {
            if (accept(op)) {
                StmtP s = mk(Stmt::Assign);
                s->op = op;
                s->lhs = lhs;
                s->e = expr();
                return s;
            }
        }
        if (lhs->k != Expr::Call) bad(lhs->line, "expression statement must be a call");
        StmtP s = mk(Stmt::Call);
        s->e = lhs;
        return s;
    }

    StmtP statement() {
        if (accept(";")) return nullptr;
        if (peek("{")) {
            StmtP s = mk(Stmt::Block);
            s->body = block();
            return s;
        }
        if (peek("@")) {
            attributes();  // statement attributes carry no meaning here
        }
        if (accept_kw("if")) return if_tail();
        if (accept_kw("return")) {
            StmtP s = mk(Stmt::Return);
            if (!peek(";")) s->e = expr();
            expect(";");
            return s;
        }
        if (accept_kw("discard")) {
            StmtP s = mk(Stmt::Discard);
            expect(";");
            return s;
        }
        if (accept_kw("break")) {
            if (accept_kw("if")) {
                StmtP s = mk(Stmt::BreakIf);
                s->e = expr();
                expect(";");
                return s;
            }
            StmtP s = mk(Stmt::Break);
            expect(";");
            return s;
        }
        if (accept_kw("continue")) {
            StmtP s = mk(Stmt::Continue);
            expect(";");
            return s;
        }
        if (accept_kw("for")) {
            StmtP s = mk(Stmt::For);
            expect("(");
            if (!peek(";")) s->init = simple_statement();
            expect(";");
            if (!peek(";")) s->e = expr();
            expect(";");
            if (!peek(")")) s->update = simple_statement();
            expect(")");
            s->body = block();
            return s;
        }
        if (accept_kw("while")) {
            StmtP s = mk(Stmt::While);
            s->e = expr();
            s->body = block();
            return s;
        }
        if (accept_kw("loop")) {
            StmtP s = mk(Stmt::Loop);
            expect("{");
            while (!accept("}")) {
                if (at_end()) bad(line(), "unterminated loop");
                if (accept_kw("continuing")) {
                    s->other = block();
                    continue;
                }
                StmtP b = statement();
                if (b) s->body.push_back(b);
            }
            return s;
        }
        if (accept_kw("switch")) {
            StmtP s = mk(Stmt::Switch);
            s->e = expr();
            expect("{");
            while (!accept("}")) {
                Stmt::Case c;
                if (accept_kw("default")) {
                    c.is_default = true;
                } else {
                    if (!accept_kw("case")) bad(line(), "expected case or default");
                    for (;;) {
                        if (accept_kw("default")) c.is_default = true;
                        else c.values.push_back(expr());
                        if (!accept(",")) break;
                        if (peek(":") || peek("{")) break;
                    }
                }
                accept(":");
                c.body = block();
                s->cases.push_back(c);
            }
            return s;
        }
        StmtP s = simple_statement();
        expect(";");
        return s;
    }

    StmtP if_tail() {
        StmtP s = mk(Stmt::If);
        s->e = expr();
        s->body = block();
        if (accept_kw("else")) {
            if (accept_kw("if")) s->other.push_back(if_tail());
            else s->other = block();
        }
        return s;
    }

    // ---- expressions, by precedence
    ExprP mkx(Expr::K k, const std::string& s, int line) {
        auto e = std::make_shared<Expr>();
        e->k = k;
        e->s = s;
        e->line = line;
        return e;
    }
    ExprP expr() { return binary(0); }

    static int prec(const std::string& op) {
        if (op == "||") return 1;
        if (op == "&&") return 2;
        if (op == "|") return 3;
        if (op == "^") return 4;
        if (op == "&") return 5;
        if (op == "==" || op == "!=") return 6;
        if (op == "<" || op == ">" || op == "<=" || op == ">=") return 7;
        if (op == "<<" || op == ">>") return 8;
        if (op == "+" || op == "-") return 9;
        if (op == "*" || op == "/" || op == "%") return 10;
        return -1;
    }
    ExprP binary(int min_prec) {
        ExprP lhs = unary();
        for (;;) {
            if (cur().t != Tk::Punct) break;
            const std::string op = cur().s;
            const int p = prec(op);
            if (p < 0 || p <= min_prec - 1 || p < min_prec) break;
            const int ln = line();
            next();
            ExprP rhs = binary(p + 1);
            ExprP e = mkx(Expr::Binary, op, ln);
            e->a = {lhs, rhs};
            lhs = e;
        }
        return lhs;
    }
    ExprP unary() {
        if (peek("-") || peek("!") || peek("~")) {
            const int ln = line();
            std::string op = cur().s;
            next();
            ExprP e = mkx(Expr::Unary, op, ln);
            e->a = {unary()};
            return e;
        }
        if (peek("&") || peek("*")) unsupported(line(), "pointers");
        return postfix(primary());
    }
    ExprP postfix(ExprP e) {
        for (;;) {
            if (accept(".")) {
                ExprP m = mkx(Expr::Member, ident(), e->line);
                m->a = {e};
                e = m;
            } else if (accept("[")) {
                ExprP ix = mkx(Expr::Index, "", e->line);
                ix->a = {e, expr()};
                expect("]");
                e = ix;
            } else {
                return e;
            }
        }
    }
    ExprP primary() {
        const int ln = line();
        if (cur().t == Tk::Int || cur().t == Tk::Float) {
            ExprP e = mkx(Expr::Lit, cur().s, ln);
            e->float_lit = cur().t == Tk::Float;
            next();
            return e;
        }
        if (accept("(")) {
            ExprP e = expr();
            expect(")");
            return e;
        }
        if (cur().t != Tk::Ident) bad(ln, "unexpected '" + cur().s + "' in expression");
        if (peek_kw("true") || peek_kw("false")) {
            ExprP e = mkx(Expr::Lit, cur().s, ln);
            next();
            return e;
        }
        const size_t save = p_;
        std::string name = ident();
        if (peek("<") && is_type_name(name)) {
            p_ = save;
            TypeExpr t = type();
            ExprP e = mkx(Expr::Call, t.name, ln);
            e->callee_type = t;
            e->templated = true;
            expect("(");
            args(e);
            return e;
        }
        if (accept("(")) {
            ExprP e = mkx(Expr::Call, name, ln);
            args(e);
            return e;
        }
        return mkx(Expr::Ident, name, ln);
    }
    void args(ExprP e) {
        while (!accept(")")) {
            e->a.push_back(expr());
            if (!accept(",")) {
                expect(")");
                break;
            }
        }
    }
    static bool is_type_name(const std::string& n) {
        return n == "vec2" || n == "vec3" || n == "vec4" || n == "array" || n.rfind("mat", 0) == 0 ||
               n == "texture_2d" || n == "ptr" || n == "atomic";
    }
};

std::shared_ptr<Module> parse(const std::string& source) {
    Parser p(lex(source));
    return p.module();
}

std::vector<std::pair<std::string, int>> entry_points(const Module& m) {
    std::vector<std::pair<std::string, int>> out;
    for (const Func& f : m.funcs)
        if (f.stage >= 0) out.emplace_back(f.name, f.stage);
    return out;
}

// ------------------------------------------------------------------------------------ types
struct Ty {
    enum K { Void, Bool, I32, U32, F32, AInt, AFloat, Vec, Mat, Struct, Arr, Tex, Samp };
    K k = Void;
    K s = Void;  // element scalar (Vec, Mat)
    int n = 0;   // vector size / matrix columns / array length
    int m = 0;   // matrix rows
    int sid = -1;
    std::shared_ptr<Ty> e;  // array element

    static Ty scalar(K k) {
        Ty t;
        t.k = k;
        return t;
    }
    static Ty vec(K s, int n) {
        Ty t;
        t.k = Vec;
        t.s = s;
        t.n = n;
        return t;
    }
    bool is_scalar() const { return k == Bool || k == I32 || k == U32 || k == F32 || k == AInt || k == AFloat; }
    bool abstract() const { return k == AInt || k == AFloat || (k == Vec && (s == AInt || s == AFloat)); }
    K scal() const { return k == Vec || k == Mat ? s : k; }
    bool numeric_int() const { K q = scal(); return q == I32 || q == U32 || q == AInt; }
    bool operator==(const Ty& o) const {
        if (k != o.k || s != o.s || n != o.n || m != o.m || sid != o.sid) return false;
        if (k == Arr) return *e == *o.e;
        return true;
    }
    bool operator!=(const Ty& o) const { return !(*this == o); }
};

static const char* scalar_c(Ty::K k) {
    switch (k) {
        case Ty::Bool: return "bool";
        case Ty::I32: return "int";
        case Ty::U32: return "unsigned";
        case Ty::F32: return "float";
        case Ty::AInt: return "int";
        case Ty::AFloat: return "float";
        default: return "void";
    }
}

// ------------------------------------------------------------------------------------ emitter
struct Val {
    std::string c;  // C++ expression
    Ty t;
    bool lit = false;     // an abstract literal (text in `text`)
    std::string text;
    double num = 0.0;
};

// A pipeline constant (f64) as a literal of the override's type, converted as naga's
// process_overrides does (WebIDL conversions): bool = value != 0 and not NaN; i32 / u32 =
// the value truncated toward zero, which must be finite and in range; f32 = the value rounded to
// nearest, finite before and after.
std::string override_literal(double value, const Ty& t, const std::string& name, int line) {
    char buf[64];
    switch (t.k) {
        case Ty::Bool: return value != 0.0 && value == value ? "true" : "false";
        case Ty::I32:
        case Ty::U32: {
            if (!std::isfinite(value)) bad(line, "pipeline constant '" + name + "' must be finite");
            const double v = std::trunc(value);
            const bool i = t.k == Ty::I32;
            if (i ? (v < -2147483648.0 || v > 2147483647.0) : (v < 0.0 || v > 4294967295.0))
                bad(line, "pipeline constant '" + name + "' is out of range of its type");
            if (i) std::snprintf(buf, sizeof buf, "(int32_t)%lldll", (long long)v);
            else std::snprintf(buf, sizeof buf, "%lluu", (unsigned long long)v);
            return buf;
        }
        case Ty::F32: {
            if (!std::isfinite(value)) bad(line, "pipeline constant '" + name + "' must be finite");
            const float f = (float)value;
            if (!std::isfinite(f)) bad(line, "pipeline constant '" + name + "' overflows f32");
            uint32_t bits;
            std::memcpy(&bits, &f, 4);
            std::snprintf(buf, sizeof buf, "__uint_as_float(0x%08xu)", bits);
            return buf;
        }
        default: unsupported(line, "an override of this type");
    }
}

class Emitter {
  public:
    Emitter(const Module& vs, const Module* fs, const Constants& vc, const Constants& fc)
        : vs_(vs), fs_(fs), vconsts_(vc), fconsts_(fc) {}

    ProgramCode run(const std::string& vs_entry, const std::string& fs_entry);

  private:
    const Module& vs_;
    const Constants& vconsts_;  // pipeline-overridable constants of the vertex / fragment stage
    const Constants& fconsts_;
    const Module* fs_;
    const Module* mod_ = nullptr;  // module being emitted
    std::string prefix_;           // name prefix of that module's declarations
    std::ostringstream decl_;      // struct definitions, uniform loaders, constants
    std::ostringstream fns_;       // helper functions (they take the JitCtx)
    std::map<std::string, Ty> const_types_, private_, uniforms_;
    std::vector<std::tuple<int, std::string, int, bool, Ty::K>> post_src_;  // location, source, comps, vector, scalar
    std::map<int, std::pair<int, int>> slot_off_;                    // location -> (first float, comps)
    std::map<int, Ty::K> slot_kind_;                                  // location -> scalar type
    struct Slot {
        int loc;
        int comps;
        int interp;  // interp_of
    };
    // flat_mask (per float) and the one mode of the other interpolated values (perspective or linear)
    void set_interpolation(const std::vector<Slot>& slots, int line) {
        pc_.flat_mask = 0;
        int mode = -1;
        for (const Slot& s : slots) {
            if (s.interp == 2) {
                const int first = slot_off_.at(s.loc).first;
                for (int k = 0; k < s.comps; ++k) pc_.flat_mask |= 1u << (first + k);
                continue;
            }
            if (mode >= 0 && s.interp != mode) unsupported(line, "linear and perspective interpolation in one program");
            mode = s.interp;
        }
        pc_.perspective = mode == 0;
    }
    std::map<std::string, int> struct_ids_;  // prefixed name -> index
    std::vector<std::pair<const StructDef*, std::string>> structs_;  // def, C name
    std::set<std::string> emitted_fns_;
    ProgramCode pc_;

    struct Var {
        Ty t;
        std::string c;
        bool mut = false;
    };
    std::vector<std::map<std::string, Var>> scopes_;
    int stage_ = -1;          // stage of the entry being emitted (-1 helper)
    bool in_entry_ = false;   // emitting an entry point's body (discard allowed)
    Ty ret_ty_;
    int tmp_ = 0;
    std::vector<std::string> loop_cont_;  // continuing label of the enclosing `loop` ("" for for/while)

    // ---- type resolution
    const StructDef* find_struct(const Module& m, const std::string& n) const {
        for (const StructDef& s : m.structs)
            if (s.name == n) return &s;
        return nullptr;
    }
    int struct_id(const Module& m, const std::string& n, int line) {
        const StructDef* sd = find_struct(m, n);
        if (!sd) bad(line, "unknown type '" + n + "'");
        const std::string cname = "S_" + prefix_ + n;
        auto it = struct_ids_.find(cname);
        if (it != struct_ids_.end()) return it->second;
        // members first (definition order in C++)
        std::vector<Ty> mt;
        for (const Member& mm : sd->members) mt.push_back(resolve(mm.ty));
        const int id = (int)structs_.size();
        structs_.emplace_back(sd, cname);
        struct_ids_[cname] = id;
        decl_ << "struct " << cname << " {";
        for (size_t i = 0; i < sd->members.size(); ++i) decl_ << " " << ctype(mt[i]) << " m_" << sd->members[i].name << ";";
        decl_ << " };\n";
        struct_member_types_[id] = mt;
        return id;
    }
    std::map<int, std::vector<Ty>> struct_member_types_;

    Ty resolve(const TypeExpr& te) {
        const std::string& n = te.name;
        auto scal = [&](const std::string& s) -> Ty::K {
            if (s == "f32") return Ty::F32;
            if (s == "i32") return Ty::I32;
            if (s == "u32") return Ty::U32;
            if (s == "bool") return Ty::Bool;
            if (s == "f16") unsupported(te.line, "f16");
            return Ty::Void;
        };
        if (Ty::K k = scal(n); k != Ty::Void) return Ty::scalar(k);
        static const std::map<std::string, std::pair<Ty::K, int>> short_vec = {
            {"vec2f", {Ty::F32, 2}}, {"vec3f", {Ty::F32, 3}}, {"vec4f", {Ty::F32, 4}}, {"vec2i", {Ty::I32, 2}},
            {"vec3i", {Ty::I32, 3}}, {"vec4i", {Ty::I32, 4}}, {"vec2u", {Ty::U32, 2}}, {"vec3u", {Ty::U32, 3}},
            {"vec4u", {Ty::U32, 4}}};
        if (auto it = short_vec.find(n); it != short_vec.end()) return Ty::vec(it->second.first, it->second.second);
        if (n == "vec2" || n == "vec3" || n == "vec4") {
            if (te.args.size() != 1) bad(te.line, n + " needs an element type");
            Ty el = resolve(te.args[0]);
            if (!el.is_scalar()) bad(te.line, "vector of non-scalar");
            return Ty::vec(el.k, n[3] - '0');
        }
        if (n.size() >= 6 && n.rfind("mat", 0) == 0 && n[4] == 'x') {
            Ty t;
            t.k = Ty::Mat;
            t.s = Ty::F32;
            t.n = n[3] - '0';
            t.m = n[5] - '0';
            if (n.size() == 7 && n[6] == 'h') unsupported(te.line, "f16 matrices");
            if (t.n < 2 || t.n > 4 || t.m < 2 || t.m > 4) bad(te.line, "bad matrix type " + n);
            return t;
        }
        if (n == "array") {
            if (te.args.size() != 1 || te.count.empty()) unsupported(te.line, "runtime-sized arrays");
            Ty t;
            t.k = Ty::Arr;
            t.e = std::make_shared<Ty>(resolve(te.args[0]));
            t.n = (int)std::strtol(te.count.c_str(), nullptr, 0);
            if (t.n <= 0) unsupported(te.line, "array length must be a positive literal");
            return t;
        }
        if (n == "texture_2d") {
            Ty t;
            t.k = Ty::Tex;
            if (te.args.size() != 1 || te.args[0].name != "f32") unsupported(te.line, "texture_2d of non-f32");
            return t;
        }
        if (n == "sampler") return Ty::scalar(Ty::Samp);
        Ty t;
        t.k = Ty::Struct;
        t.sid = struct_id(*mod_, n, te.line);
        return t;
    }

    std::string ctype(const Ty& t) const {
        switch (t.k) {
            case Ty::Bool: case Ty::I32: case Ty::U32: case Ty::F32: return scalar_c(t.k);
            case Ty::AInt: return "int";
            case Ty::AFloat: return "float";
            case Ty::Vec: return std::string("WV<") + scalar_c(t.s == Ty::AInt ? Ty::I32 : t.s == Ty::AFloat ? Ty::F32 : t.s) +
                                 "," + std::to_string(t.n) + ">";
            case Ty::Mat: return "WM<" + std::to_string(t.n) + "," + std::to_string(t.m) + ">";
            case Ty::Struct: return structs_[t.sid].second;
            case Ty::Arr: return "WA<" + ctype(*t.e) + "," + std::to_string(t.n) + ">";
            default: return "void";
        }
    }

    // ---- concretisation of abstract literals
    static Ty concrete(const Ty& t) {
        Ty r = t;
        if (r.k == Ty::AInt) r.k = Ty::I32;
        if (r.k == Ty::AFloat) r.k = Ty::F32;
        if (r.k == Ty::Vec && r.s == Ty::AInt) r.s = Ty::I32;
        if (r.k == Ty::Vec && r.s == Ty::AFloat) r.s = Ty::F32;
        return r;
    }
    // literal value of an abstract scalar as `k`
    std::string lit_as(const Val& v, Ty::K k, int line) {
        if (k == Ty::F32) {
            float f;
            if (v.t.k == Ty::AFloat) f = (float)v.num;  // f64 parse, then rounded to f32 as naga does
            else f = (float)v.num;
            uint32_t bits;
            std::memcpy(&bits, &f, 4);
            char buf[48];
            std::snprintf(buf, sizeof buf, "__uint_as_float(0x%08xu)", bits);
            return buf;
        }
        if (v.t.k == Ty::AFloat) bad(line, "float literal used as an integer");
        if (k == Ty::I32) {
            if (v.num < -2147483648.0 || v.num > 2147483647.0) bad(line, "literal out of i32 range");
            return "(int)(" + std::to_string((long long)v.num) + "ll)";
        }
        if (k == Ty::U32) {
            if (v.num < 0 || v.num > 4294967295.0) bad(line, "literal out of u32 range");
            return std::to_string((unsigned long long)v.num) + "u";
        }
        if (k == Ty::Bool) bad(line, "numeric literal used as bool");
        return v.c;
    }
    // converts `v` to type `want` when v is abstract (scalar or vector); otherwise requires equality
    Val coerce(const Val& v, const Ty& want, int line) {
        if (v.t == want) return v;
        if (v.t.k == Ty::AInt || v.t.k == Ty::AFloat) {
            if (want.is_scalar()) {
                Val r;
                r.t = want;
                r.c = lit_as(v, want.k, line);
                return r;
            }
            if (want.k == Ty::Vec) {  // abstract scalar into a vector context: keep scalar (splat handled by ops)
                Val r;
                r.t = Ty::scalar(want.s);
                r.c = lit_as(v, want.s, line);
                return r;
            }
        }
        if (v.t.k == Ty::Vec && v.t.abstract() && want.k == Ty::Vec && want.n == v.t.n) {
            Val r;
            r.t = want;
            r.c = "w_cast<" + std::string(scalar_c(want.s)) + ">(" + v.c + ")";
            return r;
        }
        bad(line, "type mismatch");
    }
    Val concretize(const Val& v, int line) {
        if (!v.t.abstract()) return v;
        return coerce(v, concrete(v.t), line);
    }

    // ---- scopes
    void push() { scopes_.emplace_back(); }
    void pop() { scopes_.pop_back(); }
    std::string declare(const std::string& name, const Ty& t, bool mut, int line) {
        if (scopes_.back().count(name)) bad(line, "'" + name + "' redeclared");
        std::string c = "u_" + name + "_" + std::to_string(tmp_++);
        scopes_.back()[name] = Var{t, c, mut};
        return c;
    }
    const Var* lookup(const std::string& name) const {
        for (auto it = scopes_.rbegin(); it != scopes_.rend(); ++it) {
            auto f = it->find(name);
            if (f != it->end()) return &f->second;
        }
        return nullptr;
    }

    // module globals reachable as identifiers
    const Global* find_global(const std::string& n) const {
        for (const Global& g : mod_->globals)
            if (g.name == n) return &g;
        return nullptr;
    }
    const Func* find_func(const std::string& n) const {
        for (const Func& f : mod_->funcs)
            if (f.name == n) return &f;
        return nullptr;
    }

    // ---- expressions
    Val ex(const ExprP& e);
    Val ex_call(const ExprP& e);
    Val construct(const Ty& t, const std::vector<Val>& args, int line);
    Val binop(const std::string& op, Val a, Val b, int line);
    Val member(const Val& base, const std::string& name, int line);
    std::string lvalue(const ExprP& e, Ty* t);

    // ---- statements
    void stmts(const std::vector<StmtP>& v, std::ostringstream& o, int ind);
    void stmt(const StmtP& s, std::ostringstream& o, int ind);

    std::string emit_function(const Func& f);
    std::string global_const(const Global& g);
    std::string uniform_loader(const Ty& t, size_t* size, size_t* align);
    void layout(const Ty& t, size_t* size, size_t* align, bool uniform);
};

static std::string pad(int n) { return std::string(2 * n, ' '); }

void Emitter::layout(const Ty& t, size_t* size, size_t* align, bool uniform) {
    auto up = [](size_t v, size_t a) { return (v + a - 1) / a * a; };
    switch (t.k) {
        case Ty::Bool: unsupported(0, "bool in a host-shareable struct");
        case Ty::I32: case Ty::U32: case Ty::F32: *size = 4; *align = 4; return;
        case Ty::Vec: *size = 4 * t.n; *align = t.n == 2 ? 8 : 16; return;
        case Ty::Mat: {
            const size_t ca = t.m == 2 ? 8 : 16, cs = 4 * t.m;
            *align = ca;
            *size = t.n * up(cs, ca);
            return;
        }
        case Ty::Arr: {
            size_t es, ea;
            layout(*t.e, &es, &ea, uniform);
            size_t stride = up(es, ea);
            if (uniform) stride = up(stride, 16);
            *align = uniform ? up(ea, 16) : ea;
            *size = stride * t.n;
            return;
        }
        case Ty::Struct: {
            size_t off = 0, al = 1;
            for (const Ty& mt : struct_member_types_[t.sid]) {
                size_t ms, ma;
                layout(mt, &ms, &ma, uniform);
                off = up(off, ma) + ms;
                al = std::max(al, ma);
            }
            if (uniform) al = up(al, 16);
            *align = al;
            *size = up(off, al);
            return;
        }
        default: unsupported(0, "type in a uniform buffer");
    }
}

// A device function that loads a value of type t from a uniform buffer at byte pointer p.
std::string Emitter::uniform_loader(const Ty& t, size_t* size, size_t* align) {
    layout(t, size, align, true);
    const std::string name = "ld_" + std::to_string(tmp_++);
    std::ostringstream o;
    auto up = [](size_t v, size_t a) { return (v + a - 1) / a * a; };
    std::function<void(const Ty&, const std::string&, size_t)> load = [&](const Ty& ty, const std::string& dst, size_t off) {
        switch (ty.k) {
            case Ty::F32: o << "  " << dst << " = __ldg(reinterpret_cast<const float*>(p + " << off << "));\n"; break;
            case Ty::I32: o << "  " << dst << " = __ldg(reinterpret_cast<const int*>(p + " << off << "));\n"; break;
            case Ty::U32: o << "  " << dst << " = __ldg(reinterpret_cast<const unsigned*>(p + " << off << "));\n"; break;
            case Ty::Vec:
                for (int i = 0; i < ty.n; ++i) load(Ty::scalar(ty.s), dst + ".c[" + std::to_string(i) + "]", off + 4 * i);
                break;
            case Ty::Mat: {
                const size_t ca = ty.m == 2 ? 8 : 16;
                for (int c = 0; c < ty.n; ++c)
                    load(Ty::vec(Ty::F32, ty.m), dst + ".col[" + std::to_string(c) + "]", off + c * up(4 * ty.m, ca));
                break;
            }
            case Ty::Arr: {
                size_t es, ea;
                layout(*ty.e, &es, &ea, true);
                const size_t stride = up(up(es, ea), 16);
                for (int i = 0; i < ty.n; ++i) load(*ty.e, dst + ".e[" + std::to_string(i) + "]", off + i * stride);
                break;
            }
            case Ty::Struct: {
                size_t o2 = off, rel = 0;
                const auto& mts = struct_member_types_[ty.sid];
                for (size_t i = 0; i < mts.size(); ++i) {
                    size_t ms, ma;
                    layout(mts[i], &ms, &ma, true);
                    rel = up(rel, ma);
                    load(mts[i], dst + ".m_" + structs_[ty.sid].first->members[i].name, o2 + rel);
                    rel += ms;
                }
                break;
            }
            default: unsupported(0, "type in a uniform buffer");
        }
    };
    o << "__device__ __forceinline__ " << ctype(t) << " " << name << "(const uint8_t* p) {\n  " << ctype(t) << " v{};\n";
    load(t, "v", 0);
    o << "  return v;\n}\n";
    decl_ << o.str();
    return name;
}

Val Emitter::ex(const ExprP& e) {
    switch (e->k) {
        case Expr::Lit: {
            Val v;
            const std::string& s = e->s;
            if (s == "true" || s == "false") {
                v.t = Ty::scalar(Ty::Bool);
                v.c = s;
                return v;
            }
            char suf = s.back();
            std::string body = s;
            if (e->float_lit) {
                if (suf == 'h') unsupported(e->line, "f16 literals");
                if (suf == 'f') {
                    body.pop_back();
                    float f = std::strtof(body.c_str(), nullptr);
                    uint32_t bits;
                    std::memcpy(&bits, &f, 4);
                    char buf[48];
                    std::snprintf(buf, sizeof buf, "__uint_as_float(0x%08xu)", bits);
                    v.t = Ty::scalar(Ty::F32);
                    v.c = buf;
                    return v;
                }
                v.t = Ty::scalar(Ty::AFloat);
                v.num = std::strtod(body.c_str(), nullptr);
                v.c = body;
                v.lit = true;
                return v;
            }
            if (suf == 'i' || suf == 'u') body.pop_back();
            const double num = (double)std::strtoull(body.c_str(), nullptr, 0);
            v.num = num;
            if (suf == 'i') {
                v.t = Ty::scalar(Ty::AInt);
                v = coerce(v, Ty::scalar(Ty::I32), e->line);
            } else if (suf == 'u') {
                v.t = Ty::scalar(Ty::AInt);
                v = coerce(v, Ty::scalar(Ty::U32), e->line);
            } else {
                v.t = Ty::scalar(Ty::AInt);
                v.c = body;
                v.lit = true;
            }
            return v;
        }
        case Expr::Ident: {
            if (const Var* var = lookup(e->s)) {
                Val v;
                v.t = var->t;
                v.c = var->c;
                return v;
            }
            if (const Global* g = find_global(e->s)) {
                Val v;
                if (g->k == Global::Const) {
                    v.c = "g_" + prefix_ + g->name + "(__tr)";
                    v.t = const_types_.at(prefix_ + g->name);
                    return v;
                }
                if (g->k == Global::Texture || g->k == Global::Sampler) {
                    v.t = Ty::scalar(g->k == Global::Texture ? Ty::Tex : Ty::Samp);
                    v.c = g->name;
                    v.text = g->name;
                    return v;
                }
                bad(e->line, "'" + e->s + "' (a uniform or private global) is only reachable from entry points");
            }
            bad(e->line, "unknown identifier '" + e->s + "'");
        }
        case Expr::Member: return member(ex(e->a[0]), e->s, e->line);
        case Expr::Index: {
            Val b = ex(e->a[0]);
            Val i = concretize(ex(e->a[1]), e->line);
            if (i.t.k != Ty::I32 && i.t.k != Ty::U32) bad(e->line, "index must be i32 or u32");
            Val r;
            if (b.t.k == Ty::Vec) {
                r.t = Ty::scalar(b.t.s);
                r.c = "w_index(" + b.c + ", " + i.c + ")";
            } else if (b.t.k == Ty::Mat) {
                r.t = Ty::vec(Ty::F32, b.t.m);
                r.c = "w_col(" + b.c + ", " + i.c + ")";
            } else if (b.t.k == Ty::Arr) {
                r.t = *b.t.e;
                r.c = "w_elem(" + b.c + ", " + i.c + ")";
            } else {
                bad(e->line, "indexing a non-composite");
            }
            r.t = concrete(r.t);
            return r;
        }
        case Expr::Unary: {
            Val a = ex(e->a[0]);
            if (a.lit && e->s == "-") {
                a.num = -a.num;
                a.c = "-" + a.c;
                return a;
            }
            a = concretize(a, e->line);
            Val r;
            r.t = a.t;
            if (e->s == "-") {
                if (a.t.scal() == Ty::U32 || a.t.scal() == Ty::Bool) bad(e->line, "negation of u32/bool");
                r.c = "w_neg(" + a.c + ")";
            } else if (e->s == "!") {
                if (a.t.scal() != Ty::Bool) bad(e->line, "! on non-bool");
                r.c = "w_lnot(" + a.c + ")";
            } else {
                if (!a.t.numeric_int()) bad(e->line, "~ on non-integer");
                r.c = "w_bnot(" + a.c + ")";
            }
            return r;
        }
        case Expr::Binary: return binop(e->s, ex(e->a[0]), ex(e->a[1]), e->line);
        case Expr::Call: return ex_call(e);
    }
    bad(e->line, "bad expression");
}

Val Emitter::member(const Val& base, const std::string& name, int line) {
    Val r;
    if (base.t.k == Ty::Struct) {
        const StructDef* sd = structs_[base.t.sid].first;
        const auto& mts = struct_member_types_[base.t.sid];
        for (size_t i = 0; i < sd->members.size(); ++i)
            if (sd->members[i].name == name) {
                r.t = mts[i];
                r.c = "(" + base.c + ").m_" + name;
                return r;
            }
        bad(line, "no member '" + name + "'");
    }
    if (base.t.k == Ty::Vec) {
        auto comp = [&](char ch) -> int {
            switch (ch) {
                case 'x': case 'r': return 0;
                case 'y': case 'g': return 1;
                case 'z': case 'b': return 2;
                case 'w': case 'a': return 3;
                default: bad(line, std::string("bad swizzle '") + name + "'");
            }
        };
        if (name.size() < 1 || name.size() > 4) bad(line, "bad swizzle");
        std::vector<int> idx;
        for (char ch : name) {
            int k = comp(ch);
            if (k >= base.t.n) bad(line, "swizzle out of range");
            idx.push_back(k);
        }
        if (idx.size() == 1) {
            r.t = Ty::scalar(base.t.s);
            r.c = "(" + base.c + ").c[" + std::to_string(idx[0]) + "]";
            return r;
        }
        r.t = Ty::vec(base.t.s, (int)idx.size());
        std::string tmp = "WV<" + std::string(scalar_c(base.t.s)) + "," + std::to_string(idx.size()) + ">{";
        // evaluate the base once
        r.c = "([&](const " + ctype(base.t) + "& s_) { return " + tmp;
        for (size_t i = 0; i < idx.size(); ++i) r.c += (i ? ", " : "") + std::string("s_.c[") + std::to_string(idx[i]) + "]";
        r.c += "}; })(" + base.c + ")";
        return r;
    }
    bad(line, "member access on a non-struct, non-vector value");
}

Val Emitter::binop(const std::string& op, Val a, Val b, int line) {
    // abstract operands take the other side's concrete scalar
    if (a.t.abstract() && !b.t.abstract()) {
        Ty want = b.t.k == Ty::Mat ? Ty::scalar(Ty::F32) : (b.t.k == Ty::Vec ? Ty::scalar(b.t.s) : b.t);
        if (op == "<<" || op == ">>") want = Ty::scalar(Ty::I32);
        a = a.t.k == Ty::Vec ? coerce(a, Ty::vec(want.k, a.t.n), line) : coerce(a, want, line);
    } else if (b.t.abstract() && !a.t.abstract()) {
        Ty want = a.t.k == Ty::Mat ? Ty::scalar(Ty::F32) : (a.t.k == Ty::Vec ? Ty::scalar(a.t.s) : a.t);
        if (op == "<<" || op == ">>") want = Ty::scalar(Ty::U32);
        b = b.t.k == Ty::Vec ? coerce(b, Ty::vec(want.k, b.t.n), line) : coerce(b, want, line);
    } else if (a.t.abstract() && b.t.abstract()) {
        const bool fl = a.t.scal() == Ty::AFloat || b.t.scal() == Ty::AFloat;
        const Ty::K k = fl ? Ty::F32 : Ty::I32;
        a = a.t.k == Ty::Vec ? coerce(a, Ty::vec(k, a.t.n), line) : coerce(a, Ty::scalar(k), line);
        b = b.t.k == Ty::Vec ? coerce(b, Ty::vec(k, b.t.n), line) : coerce(b, Ty::scalar(k), line);
    }
    Val r;
    auto same_scalar = [&]() {
        if (a.t.scal() != b.t.scal()) bad(line, "operand types differ in '" + op + "'");
    };
    if (op == "&&" || op == "||") {
        if (a.t.k != Ty::Bool || b.t.k != Ty::Bool) bad(line, op + " needs bool operands");
        r.t = a.t;
        r.c = "(" + a.c + " " + op + " " + b.c + ")";
        return r;
    }
    if (op == "==" || op == "!=" || op == "<" || op == "<=" || op == ">" || op == ">=") {
        same_scalar();
        if (a.t.k == Ty::Mat || a.t.k == Ty::Struct || a.t.k == Ty::Arr) bad(line, "comparison of composites");
        if (a.t.k == Ty::Vec && b.t.k == Ty::Vec && a.t.n != b.t.n) bad(line, "vector sizes differ");
        static const std::map<std::string, std::string> f = {{"==", "w_eq"}, {"!=", "w_ne"}, {"<", "w_lt"},
                                                             {"<=", "w_le"}, {">", "w_gt"},  {">=", "w_ge"}};
        r.t = a.t.k == Ty::Vec ? Ty::vec(Ty::Bool, a.t.n) : (b.t.k == Ty::Vec ? Ty::vec(Ty::Bool, b.t.n) : Ty::scalar(Ty::Bool));
        r.c = f.at(op) + "(" + a.c + ", " + b.c + ")";
        return r;
    }
    if (op == "*" && a.t.k == Ty::Mat) {
        if (b.t.k == Ty::Vec) {
            if (b.t.n != a.t.n || b.t.s != Ty::F32) bad(line, "matrix * vector size mismatch");
            r.t = Ty::vec(Ty::F32, a.t.m);
            r.c = "w_mulmv(" + a.c + ", " + b.c + ")";
            return r;
        }
        if (b.t.k == Ty::F32) {
            r.t = a.t;
            r.c = "w_mul(" + a.c + ", " + b.c + ")";
            return r;
        }
        unsupported(line, "matrix * matrix (naga-cranelift/src/expression/binary.rs:273-325 multiplies matrices by vectors and scalars)");
    }
    if (op == "*" && b.t.k == Ty::Mat) {
        if (a.t.k == Ty::F32) {
            r.t = b.t;
            r.c = "w_mul(" + a.c + ", " + b.c + ")";
            return r;
        }
        unsupported(line, "vector * matrix");
    }
    if ((op == "+" || op == "-") && a.t.k == Ty::Mat) {
        if (b.t != a.t) bad(line, "matrix operand mismatch");
        r.t = a.t;
        r.c = std::string(op == "+" ? "w_add(" : "w_sub(") + a.c + ", " + b.c + ")";
        return r;
    }
    static const std::map<std::string, std::string> arith = {
        {"+", "w_add"}, {"-", "w_sub"}, {"*", "w_mul"}, {"/", "w_div"}, {"%", "w_rem"},
        {"&", "w_and"}, {"|", "w_or"},  {"^", "w_xor"}, {"<<", "w_shl"}, {">>", "w_shr"}};
    auto it = arith.find(op);
    if (it == arith.end()) bad(line, "unknown operator " + op);
    if (a.t.k == Ty::Struct || b.t.k == Ty::Struct || a.t.k == Ty::Arr || b.t.k == Ty::Arr) bad(line, "arithmetic on composites");
    if (op == "<<" || op == ">>") {
        if (!a.t.numeric_int() || b.t.scal() != Ty::U32) bad(line, "shift needs an integer and a u32 amount");
        r.t = a.t;
        r.c = it->second + "(" + a.c + ", " + b.c + ")";
        return r;
    }
    same_scalar();
    if (a.t.k == Ty::Vec && b.t.k == Ty::Vec && a.t.n != b.t.n) bad(line, "vector sizes differ");
    const Ty::K s = a.t.scal();
    if ((op == "&" || op == "|" || op == "^") && s == Ty::F32) bad(line, "bitwise op on f32");
    if ((op == "+" || op == "-" || op == "*" || op == "/" || op == "%") && s == Ty::Bool) bad(line, "arithmetic on bool");
    r.t = a.t.k == Ty::Vec ? a.t : b.t;
    if (op == "/" || op == "%") r.c = it->second + "(" + a.c + ", " + b.c + ", __tr)";
    else r.c = it->second + "(" + a.c + ", " + b.c + ")";
    return r;
}

Val Emitter::construct(const Ty& t, const std::vector<Val>& args0, int line) {
    Val r;
    r.t = t;
    std::vector<Val> args = args0;
    if (t.is_scalar()) {  // conversion
        if (args.size() != 1) bad(line, "scalar constructor takes one argument");
        Val a = args[0];
        if (a.t.abstract()) {
            if (a.t.k == Ty::AFloat && t.k != Ty::F32 && t.k != Ty::Bool) {
                a = coerce(a, Ty::scalar(Ty::F32), line);
            } else if (t.k != Ty::Bool) {
                return coerce(a, t, line);
            } else {
                a = concretize(a, line);
            }
        }
        if (!a.t.is_scalar()) bad(line, "scalar conversion of a composite");
        static const std::map<Ty::K, std::string> f = {{Ty::F32, "w_f32"}, {Ty::I32, "w_i32"}, {Ty::U32, "w_u32"},
                                                       {Ty::Bool, "w_bool"}};
        r.c = f.at(t.k) + "(" + a.c + ")";
        return r;
    }
    if (t.k == Ty::Vec) {
        if (args.empty()) {
            r.c = ctype(t) + "{}";
            return r;
        }
        if (args.size() == 1 && args[0].t.k == Ty::Vec) {  // conversion
            Val a = args[0].t.abstract() ? coerce(args[0], Ty::vec(t.s, args[0].t.n), line) : args[0];
            if (a.t.n != t.n) bad(line, "vector conversion size mismatch");
            static const std::map<Ty::K, std::string> f = {{Ty::F32, "w_f32"}, {Ty::I32, "w_i32"}, {Ty::U32, "w_u32"},
                                                           {Ty::Bool, "w_bool"}};
            r.c = f.at(t.s) + "(" + a.c + ")";
            return r;
        }
        if (args.size() == 1) {  // splat
            Val a = args[0].t.abstract() ? coerce(args[0], Ty::scalar(t.s), line) : args[0];
            if (a.t.k != t.s) bad(line, "splat of a different scalar type");
            r.c = "w_splat<" + std::string(scalar_c(t.s)) + "," + std::to_string(t.n) + ">(" + a.c + ")";
            return r;
        }
        std::vector<std::string> comps;
        for (Val a : args) {
            if (a.t.abstract()) a = a.t.k == Ty::Vec ? coerce(a, Ty::vec(t.s, a.t.n), line) : coerce(a, Ty::scalar(t.s), line);
            if (a.t.scal() != t.s) bad(line, "vector component type mismatch");
            if (a.t.k == Ty::Vec) {
                // compose from a vector: naga-cranelift panics here (expression/compose.rs:229-243);
                // WebGPU semantics are a plain component copy
                const std::string tmpn = "cv" + std::to_string(tmp_++);
                for (int i = 0; i < a.t.n; ++i) comps.push_back("(" + a.c + ").c[" + std::to_string(i) + "]");
            } else {
                comps.push_back(a.c);
            }
        }
        if ((int)comps.size() != t.n) bad(line, "vector constructor component count");
        r.c = ctype(t) + "{";
        for (size_t i = 0; i < comps.size(); ++i) r.c += (i ? ", " : "") + comps[i];
        r.c += "}";
        return r;
    }
    if (t.k == Ty::Mat) {
        if (args.empty()) {
            r.c = ctype(t) + "{}";
            return r;
        }
        std::vector<std::string> cols;
        if ((int)args.size() == t.n) {
            for (Val a : args) {
                if (a.t.abstract()) a = coerce(a, Ty::vec(Ty::F32, a.t.n), line);
                if (a.t != Ty::vec(Ty::F32, t.m)) bad(line, "matrix column type mismatch");
                cols.push_back(a.c);
            }
        } else if ((int)args.size() == t.n * t.m) {
            for (int c = 0; c < t.n; ++c) {
                std::string col = "WV<float," + std::to_string(t.m) + ">{";
                for (int k = 0; k < t.m; ++k) {
                    Val a = args[c * t.m + k];
                    if (a.t.abstract()) a = coerce(a, Ty::scalar(Ty::F32), line);
                    if (a.t.k != Ty::F32) bad(line, "matrix element type mismatch");
                    col += (k ? ", " : "") + a.c;
                }
                cols.push_back(col + "}");
            }
        } else {
            bad(line, "matrix constructor argument count");
        }
        r.c = ctype(t) + "{{";
        for (size_t i = 0; i < cols.size(); ++i) r.c += (i ? ", " : "") + cols[i];
        r.c += "}}";
        return r;
    }
    if (t.k == Ty::Struct) {
        const auto& mts = struct_member_types_[t.sid];
        if (args.empty()) {
            r.c = ctype(t) + "{}";
            return r;
        }
        if (args.size() != mts.size()) bad(line, "struct constructor argument count");
        r.c = ctype(t) + "{";
        for (size_t i = 0; i < args.size(); ++i) {
            Val a = args[i].t.abstract() ? coerce(args[i], mts[i], line) : args[i];
            if (a.t != mts[i]) bad(line, "struct member " + std::to_string(i) + " type mismatch");
            r.c += (i ? ", " : "") + a.c;
        }
        r.c += "}";
        return r;
    }
    if (t.k == Ty::Arr) {
        if (args.empty()) {
            r.c = ctype(t) + "{}";
            return r;
        }
        if ((int)args.size() != t.n) bad(line, "array constructor element count");
        r.c = ctype(t) + "{{";
        for (size_t i = 0; i < args.size(); ++i) {
            Val a = args[i].t.abstract() ? coerce(args[i], *t.e, line) : args[i];
            if (a.t != *t.e) bad(line, "array element type mismatch");
            r.c += (i ? ", " : "") + a.c;
        }
        r.c += "}}";
        return r;
    }
    bad(line, "cannot construct this type");
}

Val Emitter::ex_call(const ExprP& e) {
    std::vector<Val> args;
    for (const ExprP& a : e->a) args.push_back(ex(a));
    const std::string& n = e->s;
    if (e->templated) return construct(resolve(e->callee_type), args, e->line);
    // inferred-element constructors (vec4(...), mat4x4(...))
    if (n == "vec2" || n == "vec3" || n == "vec4") {
        Ty::K s = Ty::Void;
        for (const Val& a : args) {
            const Ty::K k = a.t.scal();
            if (k != Ty::AInt && k != Ty::AFloat) s = k;
        }
        if (s == Ty::Void) {
            bool fl = false;
            for (const Val& a : args) fl = fl || a.t.scal() == Ty::AFloat;
            s = fl ? Ty::F32 : Ty::I32;
        }
        return construct(Ty::vec(s, n[3] - '0'), args, e->line);
    }
    if (n == "select") {
        if (args.size() != 3) bad(e->line, "select takes three arguments");
        Val f = args[0], t = args[1], c = args[2];
        if (f.t.abstract() && !t.t.abstract()) f = coerce(f, t.t, e->line);
        if (t.t.abstract() && !f.t.abstract()) t = coerce(t, f.t, e->line);
        f = concretize(f, e->line);
        t = concretize(t, e->line);
        if (f.t != t.t) bad(e->line, "select operand types differ");
        if (c.t.scal() != Ty::Bool) bad(e->line, "select condition must be bool");
        Val r;
        r.t = f.t;
        r.c = "w_select(" + f.c + ", " + t.c + ", " + c.c + ")";
        return r;
    }
    if (n == "textureSample") {
        if (stage_ != 1) bad(e->line, "textureSample outside the fragment stage");
        if (args.size() != 3) unsupported(e->line, "textureSample with an offset or array index");
        if (args[0].t.k != Ty::Tex || args[1].t.k != Ty::Samp) bad(e->line, "textureSample(texture, sampler, coords)");
        const Global* tg = find_global(args[0].text);
        const Global* sg = find_global(args[1].text);
        if (pc_.tex_group >= 0 && (pc_.tex_group != tg->group || pc_.tex_binding != tg->binding))
            unsupported(e->line, "more than one sampled texture");
        if (pc_.samp_group >= 0 && (pc_.samp_group != sg->group || pc_.samp_binding != sg->binding))
            unsupported(e->line, "more than one sampler");
        pc_.tex_group = tg->group;
        pc_.tex_binding = tg->binding;
        pc_.samp_group = sg->group;
        pc_.samp_binding = sg->binding;
        Val uv = args[2];
        if (uv.t.abstract()) uv = coerce(uv, Ty::vec(Ty::F32, 2), e->line);
        if (uv.t != Ty::vec(Ty::F32, 2)) bad(e->line, "textureSample coordinates must be vec2f");
        Val r;
        r.t = Ty::vec(Ty::F32, 4);
        r.c = "w_sample(*__c.d, " + uv.c + ")";
        return r;
    }
    static const std::set<std::string> math = {"abs", "acos", "asin", "atan", "atan2", "ceil", "clamp", "cos", "cross",
                                                "degrees", "distance", "dot", "exp", "exp2", "floor", "fract", "inverseSqrt",
                                                "length", "log", "log2", "max", "min", "mix", "normalize", "pow", "radians",
                                                "reflect", "round", "sign", "sin", "smoothstep", "sqrt", "step", "tan",
                                                "trunc", "fma", "saturate", "transpose", "determinant", "dpdx", "dpdy",
                                                "fwidth", "textureLoad", "textureSampleLevel", "textureSampleBias",
                                                "textureDimensions", "all", "any", "arrayLength"};
    if (math.count(n))
        unsupported(e->line, "builtin function " + n + " (naga-cranelift implements none of the math builtins: "
                             "expression/math.rs:21-24)");
    if (n == "f32" || n == "i32" || n == "u32" || n == "bool" || n == "vec2f" || n == "vec3f" || n == "vec4f" ||
        n == "vec2i" || n == "vec3i" || n == "vec4i" || n == "vec2u" || n == "vec3u" || n == "vec4u" ||
        (n.rfind("mat", 0) == 0 && n.size() >= 6 && n[4] == 'x')) {
        TypeExpr te;
        te.name = n;
        te.line = e->line;
        return construct(resolve(te), args, e->line);
    }
    if (find_struct(*mod_, n)) {
        TypeExpr te;
        te.name = n;
        te.line = e->line;
        return construct(resolve(te), args, e->line);
    }
    const Func* f = find_func(n);
    if (!f) bad(e->line, "unknown function '" + n + "'");
    if (f->stage >= 0) bad(e->line, "calling an entry point");
    if (f->params.size() != args.size()) bad(e->line, "argument count of " + n);
    const std::string fname = emit_function(*f);
    Val r;
    r.t = f->has_ret ? concrete(resolve(f->ret)) : Ty();
    r.c = fname + "(__c, __tr";
    for (size_t i = 0; i < args.size(); ++i) {
        Ty pt = resolve(f->params[i].ty);
        Val a = args[i].t.abstract() ? coerce(args[i], pt, e->line) : args[i];
        if (a.t != pt) bad(e->line, "argument " + std::to_string(i) + " of " + n + " has the wrong type");
        r.c += ", " + a.c;
    }
    r.c += ")";
    return r;
}

std::string Emitter::lvalue(const ExprP& e, Ty* t) {
    switch (e->k) {
        case Expr::Ident: {
            const Var* v = lookup(e->s);
            if (!v) {
                const Global* g = find_global(e->s);
                if (g && g->k == Global::Private)
                    bad(e->line, "'" + e->s + "' (a private global) is only reachable from entry points");
                bad(e->line, "cannot assign to '" + e->s + "'");
            }
            if (!v->mut) bad(e->line, "'" + e->s + "' is not a var");
            *t = v->t;
            return v->c;
        }
        case Expr::Member: {
            Ty bt;
            std::string b = lvalue(e->a[0], &bt);
            Val base;
            base.t = bt;
            base.c = b;
            if (bt.k == Ty::Vec && e->s.size() != 1) unsupported(e->line, "assignment to a multi-component swizzle");
            Val m = member(base, e->s, e->line);
            *t = m.t;
            return m.c;
        }
        case Expr::Index: {
            Ty bt;
            std::string b = lvalue(e->a[0], &bt);
            Val i = concretize(ex(e->a[1]), e->line);
            if (bt.k == Ty::Vec) {
                *t = Ty::scalar(bt.s);
                return "w_index_ref(" + b + ", " + i.c + ")";
            }
            if (bt.k == Ty::Mat) {
                *t = Ty::vec(Ty::F32, bt.m);
                return "w_col_ref(" + b + ", " + i.c + ")";
            }
            if (bt.k == Ty::Arr) {
                *t = *bt.e;
                return "w_elem_ref(" + b + ", " + i.c + ")";
            }
            bad(e->line, "indexing a non-composite");
        }
        default: bad(e->line, "not assignable");
    }
}

void Emitter::stmts(const std::vector<StmtP>& v, std::ostringstream& o, int ind) {
    for (const StmtP& s : v) stmt(s, o, ind);
}

void Emitter::stmt(const StmtP& s, std::ostringstream& o, int ind) {
    const std::string P = pad(ind);
    switch (s->k) {
        case Stmt::Let:
        case Stmt::Const:
        case Stmt::Var: {
            Ty t;
            std::string init;
            if (s->e) {
                Val v = ex(s->e);
                if (s->has_type) {
                    t = resolve(s->ty);
                    v = v.t.abstract() ? coerce(v, t, s->line) : v;
                    if (v.t != t) bad(s->line, "initializer type of '" + s->name + "'");
                } else {
                    v = concretize(v, s->line);
                    t = v.t;
                }
                init = v.c;
            } else {
                t = resolve(s->ty);
                init = ctype(t) + "{}";
            }
            const std::string c = declare(s->name, t, s->k == Stmt::Var, s->line);
            o << P << (s->k == Stmt::Var ? "" : "const ") << ctype(t) << " " << c << " = " << init << ";\n";
            return;
        }
        case Stmt::Assign: {
            Ty t;
            const std::string lv = lvalue(s->lhs, &t);
            Val v = ex(s->e);
            if (s->op == "=") {
                v = v.t.abstract() ? coerce(v, t, s->line) : v;
                if (v.t != t) bad(s->line, "assigned value type mismatch");
                o << P << lv << " = " << v.c << ";\n";
            } else {
                Val cur;
                cur.t = t;
                cur.c = lv;
                Val r = binop(s->op.substr(0, s->op.size() - 1), cur, v, s->line);
                if (r.t != t) bad(s->line, "compound assignment changes the type");
                o << P << lv << " = " << r.c << ";\n";
            }
            return;
        }
        case Stmt::Incr:
        case Stmt::Decr: {
            Ty t;
            const std::string lv = lvalue(s->lhs, &t);
            if (t.k != Ty::I32 && t.k != Ty::U32) bad(s->line, "++/-- on a non-integer");
            o << P << lv << " = " << (s->k == Stmt::Incr ? "w_add(" : "w_sub(") << lv << ", (" << ctype(t) << ")1);\n";
            return;
        }
        case Stmt::If: {
            Val c = ex(s->e);
            if (c.t.k != Ty::Bool) bad(s->line, "if condition must be bool");
            o << P << "if (" << c.c << ") {\n";
            push();
            stmts(s->body, o, ind + 1);
            pop();
            o << P << "}";
            if (!s->other.empty()) {
                o << " else {\n";
                push();
                stmts(s->other, o, ind + 1);
                pop();
                o << P << "}";
            }
            o << "\n";
            return;
        }
        case Stmt::For: {
            push();
            o << P << "{\n";
            if (s->init) stmt(s->init, o, ind + 1);
            std::string cond = "true";
            if (s->e) {
                Val c = ex(s->e);
                if (c.t.k != Ty::Bool) bad(s->line, "for condition must be bool");
                cond = c.c;
            }
            std::ostringstream upd;
            if (s->update) stmt(s->update, upd, 0);
            std::string u = upd.str();
            while (!u.empty() && (u.back() == '\n' || u.back() == ';')) u.pop_back();
            o << pad(ind + 1) << "for (; " << cond << "; " << "[&]() { " << u << "; }()) {\n";
            loop_cont_.push_back("");
            push();
            stmts(s->body, o, ind + 2);
            pop();
            loop_cont_.pop_back();
            o << pad(ind + 1) << "}\n" << P << "}\n";
            pop();
            return;
        }
        case Stmt::While: {
            Val c = ex(s->e);
            if (c.t.k != Ty::Bool) bad(s->line, "while condition must be bool");
            o << P << "while (" << c.c << ") {\n";
            loop_cont_.push_back("");
            push();
            stmts(s->body, o, ind + 1);
            pop();
            loop_cont_.pop_back();
            o << P << "}\n";
            return;
        }
        case Stmt::Loop: {
            const std::string label = "cont_" + std::to_string(tmp_++);
            o << P << "for (;;) {\n";
            loop_cont_.push_back(label);
            push();
            o << pad(ind + 1) << "{\n";
            push();
            stmts(s->body, o, ind + 2);
            pop();
            o << pad(ind + 1) << "}\n";
            o << pad(ind + 1) << label << ": ;\n";
            stmts(s->other, o, ind + 1);
            pop();
            loop_cont_.pop_back();
            o << P << "}\n";
            return;
        }
        case Stmt::Break: o << P << "break;\n"; return;
        case Stmt::BreakIf: {
            Val c = ex(s->e);
            if (c.t.k != Ty::Bool) bad(s->line, "break if condition must be bool");
            o << P << "if (" << c.c << ") break;\n";
            return;
        }
        case Stmt::Continue:
            if (loop_cont_.empty()) bad(s->line, "continue outside a loop");
            if (loop_cont_.back().empty()) o << P << "continue;\n";
            else o << P << "goto " << loop_cont_.back() << ";\n";
            return;
        case Stmt::Return: {
            if (!s->e) {
                if (ret_ty_.k != Ty::Void) bad(s->line, "return without a value");
                o << P << "return;\n";
                return;
            }
            Val v = ex(s->e);
            v = v.t.abstract() ? coerce(v, ret_ty_, s->line) : v;
            if (v.t != ret_ty_) bad(s->line, "returned value type mismatch");
            o << P << "return " << v.c << ";\n";
            return;
        }
        case Stmt::Discard:
            if (stage_ != 1) bad(s->line, "discard outside the fragment stage");
            if (!in_entry_) unsupported(s->line, "discard inside a helper function");
            pc_.may_discard = true;
            o << P << "{ __c.kill = true; return " << ctype(ret_ty_) << "{}; }\n";
            return;
        case Stmt::Switch: {
            Val sel = concretize(ex(s->e), s->line);
            if (sel.t.k != Ty::I32 && sel.t.k != Ty::U32) bad(s->line, "switch selector must be i32 or u32");
            o << P << "switch (" << sel.c << ") {\n";
            for (const Stmt::Case& c : s->cases) {
                for (const ExprP& v : c.values) {
                    Val cv = ex(v);
                    if (!cv.lit && !(cv.t == sel.t)) bad(s->line, "case value type");
                    o << P << "case " << (cv.lit ? lit_as(cv, sel.t.k, s->line) : cv.c) << ":\n";
                }
                if (c.is_default) o << P << "default:\n";
                o << P << "{\n";
                push();
                loop_cont_.push_back(loop_cont_.empty() ? "" : loop_cont_.back());
                stmts(c.body, o, ind + 1);
                loop_cont_.pop_back();
                pop();
                o << P << "break; }\n";
            }
            o << P << "}\n";
            return;
        }
        case Stmt::Block:
            o << P << "{\n";
            push();
            stmts(s->body, o, ind + 1);
            pop();
            o << P << "}\n";
            return;
        case Stmt::Call: {
            Val v = ex(s->e);
            o << P << "(void)(" << v.c << ");\n";
            return;
        }
    }
}

std::string Emitter::emit_function(const Func& f) {
    const std::string name = "fn_" + prefix_ + f.name;
    if (emitted_fns_.count(name)) return name;
    emitted_fns_.insert(name);
    auto saved_scopes = scopes_;
    const Ty saved_ret = ret_ty_;
    const bool saved_entry = in_entry_;
    scopes_.clear();
    push();
    in_entry_ = false;
    ret_ty_ = f.has_ret ? concrete(resolve(f.ret)) : Ty();
    std::ostringstream o;
    o << "__device__ " << ctype(ret_ty_) << " " << name << "(JitCtx& __c, bool& __tr";
    for (const Member& p : f.params) {
        Ty t = resolve(p.ty);
        o << ", " << ctype(t) << " " << declare(p.name, t, false, f.line);
    }
    o << ") {\n";
    stmts(f.body, o, 1);
    if (ret_ty_.k != Ty::Void) o << "  return " << ctype(ret_ty_) << "{};\n";
    o << "}\n";
    fns_ << o.str();
    scopes_ = saved_scopes;
    ret_ty_ = saved_ret;
    in_entry_ = saved_entry;
    return name;
}

// ---------------------------------------------------------------------------- entry points
namespace {
int builtin_of(const std::vector<Attr>& attrs, std::string* name) {
    for (const Attr& a : attrs)
        if (a.name == "builtin" && !a.args.empty()) {
            *name = a.args[0];
            return 1;
        }
    return 0;
}
int location_of(const std::vector<Attr>& attrs) {
    for (const Attr& a : attrs)
        if (a.name == "location" && !a.args.empty()) return std::atoi(a.args[0].c_str());
    return -1;
}
// @interpolate(type[, sampling]) of an inter-stage value: 0 = perspective, 1 = linear, 2 = flat.
// Without the attribute naga applies the default: perspective for floats, flat for integers
// (Binding::apply_default_interpolation).  The sampling must fit the type as naga validates it (flat: first / either;
// perspective / linear: center / centroid / sample); the reference interpolates every sampling
// the same way (fragment.rs:278-378, FlatSampling at :395-405).
int interp_of(const std::vector<Attr>& attrs, int line, bool integer) {
    for (const Attr& a : attrs)
        if (a.name == "interpolate") {
            if (a.args.empty() || a.args.size() > 2) bad(line, "@interpolate takes a type and an optional sampling");
            int type = -1;
            if (a.args[0] == "perspective") type = 0;
            else if (a.args[0] == "linear") type = 1;
            else if (a.args[0] == "flat") type = 2;
            else bad(line, "unknown interpolation type '" + a.args[0] + "'");
            if (a.args.size() == 2) {
                const std::string& s = a.args[1];
                const bool flat_ok = s == "first" || s == "either";
                const bool other_ok = s == "center" || s == "centroid" || s == "sample";
                if (!flat_ok && !other_ok) bad(line, "unknown interpolation sampling '" + s + "'");
                if ((type == 2) != flat_ok) bad(line, "sampling '" + s + "' does not apply to " + a.args[0] + " interpolation");
            }
            return type;
        }
    return integer ? 2 : 0;
}
}  // namespace

ProgramCode Emitter::run(const std::string& vs_entry, const std::string& fs_entry) {
    for (auto& g : pc_.input_loc) g = -1;
    std::ostringstream body;
    std::vector<Slot> slots;  // varyings in location order

    // ---------- vertex stage
    mod_ = &vs_;
    prefix_ = "v_";
    const Func* vf = nullptr;
    for (const Func& f : vs_.funcs)
        if (f.name == vs_entry && f.stage == 0) vf = &f;
    if (!vf) throw Error("no @vertex entry point '" + vs_entry + "'", false);
    auto emit_consts = [&](const Module& m, const Constants& consts) {
        for (const Global& g : m.globals)
            if (g.k == Global::Const) {
                scopes_.clear();
                push();
                // an override takes the pipeline's value when one is given under its key (its
                // @id, else its name), else its initializer (process_overrides)
                const Constants::const_iterator given =
                    g.is_override ? consts.find(g.override_id >= 0 ? std::to_string(g.override_id) : g.name)
                                  : consts.end();
                Ty t;
                Val v;
                if (given != consts.end()) {
                    t = g.has_type ? resolve(g.ty) : concretize(ex(g.init), g.line).t;
                    v.t = t;
                    v.c = override_literal(given->second, t, g.name, g.line);
                } else {
                    if (!g.init) bad(g.line, "override '" + g.name + "' has no value: the pipeline gives none and it has no initializer");
                    v = ex(g.init);
                    if (g.has_type) {
                        t = resolve(g.ty);
                        v = v.t.abstract() ? coerce(v, t, g.line) : v;
                    } else {
                        v = concretize(v, g.line);
                        t = v.t;
                    }
                }
                const_types_[prefix_ + g.name] = t;
                decl_ << "__device__ __forceinline__ " << ctype(t) << " g_" << prefix_ << g.name << "(bool& __tr) { return "
                      << v.c << "; }\n";
            }
    };
    emit_consts(vs_, vconsts_);

    // the context: private globals, uniform values, the draw
    auto ctx_members = [&](const Module& m, std::ostringstream& members, std::ostringstream& init) {
        for (const Global& g : m.globals) {
            if (g.k == Global::Private) {
                Ty t = g.has_type ? resolve(g.ty) : Ty();
                std::string iv;
                if (g.init) {
                    scopes_.clear();
                    push();
                    Val v = ex(g.init);
                    if (!g.has_type) {
                        v = concretize(v, g.line);
                        t = v.t;
                    } else {
                        v = v.t.abstract() ? coerce(v, t, g.line) : v;
                    }
                    iv = v.c;
                } else {
                    iv = ctype(t) + "{}";
                }
                members << "  " << ctype(t) << " p_" << prefix_ << g.name << ";\n";
                init << "  __c.p_" << prefix_ << g.name << " = " << iv << ";\n";
                private_[prefix_ + g.name] = t;
            } else if (g.k == Global::Uniform) {
                if (!g.has_type) bad(g.line, "uniform without a type");
                Ty t = resolve(g.ty);
                size_t size, align;
                const std::string ld = uniform_loader(t, &size, &align);
                pc_.uniform_size[g.group][g.binding] = std::max<uint32_t>(pc_.uniform_size[g.group][g.binding], (uint32_t)size);
                members << "  " << ctype(t) << " q_" << prefix_ << g.name << ";\n";
                init << "  __c.q_" << prefix_ << g.name << " = " << ld << "(d.uniform[" << g.group << "][" << g.binding
                     << "]);\n";
                uniforms_[prefix_ + g.name] = t;
            }
        }
    };

    // entry-point scopes see private and uniform globals through __c
    auto push_globals = [&](const Module& m) {
        push();
        for (const Global& g : m.globals) {
            if (g.k == Global::Private) scopes_.back()[g.name] = Var{private_[prefix_ + g.name], "__c.p_" + prefix_ + g.name, true};
            if (g.k == Global::Uniform) scopes_.back()[g.name] = Var{uniforms_[prefix_ + g.name], "__c.q_" + prefix_ + g.name, false};
        }
    };

    std::ostringstream vmembers, vinit;
    ctx_members(vs_, vmembers, vinit);

    std::ostringstream vw;
    {
        stage_ = 0;
        in_entry_ = true;
        scopes_.clear();
        push_globals(vs_);
        push();
        std::ostringstream pre;  // inputs
        int ninput = 0;
        auto input = [&](const Member& p, const Ty& t, const std::string& dst) {
            std::string bname;
            if (builtin_of(p.attrs, &bname)) {
                if (bname == "vertex_index") {
                    if (t.k != Ty::U32) bad(vf->line, "vertex_index must be u32");
                    pre << "  " << dst << " = vertex;\n";
                } else if (bname == "instance_index") {
                    if (t.k != Ty::U32) bad(vf->line, "instance_index must be u32");
                    pre << "  " << dst << " = instance;\n";
                } else {
                    unsupported(vf->line, "vertex input builtin " + bname);
                }
                return;
            }
            const int loc = location_of(p.attrs);
            if (loc < 0 || loc >= 16) bad(vf->line, "vertex input '" + p.name + "' needs @location(0..15)");
            int comps = 1;
            Ty::K sk = t.k;
            if (t.k == Ty::Vec) {
                comps = t.n;
                sk = t.s;
            }
            if (sk != Ty::F32 && sk != Ty::I32 && sk != Ty::U32) unsupported(vf->line, "vertex input type");
            if (ninput >= 16) bad(vf->line, "too many vertex inputs");
            pc_.input_loc[ninput] = loc;
            pc_.input_comps[ninput] = comps;
            pc_.input_kind[ninput] = sk == Ty::F32 ? 0 : sk == Ty::I32 ? 1 : 2;
            ++ninput;
            pre << "  { float a_[4]; if (!fetch_attr(d, " << loc << ", " << comps << ", vertex, instance, a_, err)) return false;\n";
            for (int i = 0; i < comps; ++i) {
                const std::string comp = t.k == Ty::Vec ? dst + ".c[" + std::to_string(i) + "]" : dst;
                const char* conv = sk == Ty::F32 ? "" : sk == Ty::I32 ? "__float_as_int" : "__float_as_uint";
                pre << "    " << comp << " = " << conv << "(a_[" << i << "]);\n";
            }
            pre << "  }\n";
        };
        std::ostringstream decls;
        for (const Member& p : vf->params) {
            Ty t = resolve(p.ty);
            const std::string c = declare(p.name, t, false, vf->line);
            decls << "  " << ctype(t) << " " << c << "{};\n";
            if (t.k == Ty::Struct) {
                const StructDef* sd = structs_[t.sid].first;
                const auto& mts = struct_member_types_[t.sid];
                for (size_t i = 0; i < sd->members.size(); ++i) input(sd->members[i], mts[i], c + ".m_" + sd->members[i].name);
            } else {
                input(p, t, c);
            }
        }
        pc_.num_inputs = ninput;
        if (!vf->has_ret) bad(vf->line, "vertex entry point without a return value");
        ret_ty_ = resolve(vf->ret);
        // output layout
        std::ostringstream post;
        bool have_pos = false;
        auto output = [&](const std::vector<Attr>& attrs, const Ty& t, const std::string& src) {
            std::string bname;
            if (builtin_of(attrs, &bname)) {
                if (bname != "position") unsupported(vf->line, "vertex output builtin " + bname);
                if (t != Ty::vec(Ty::F32, 4)) bad(vf->line, "position must be vec4f");
                post << "  pos = V4{" << src << ".c[0], " << src << ".c[1], " << src << ".c[2], " << src << ".c[3]};\n";
                have_pos = true;
                return;
            }
            const int loc = location_of(attrs);
            if (loc < 0) bad(vf->line, "vertex output needs @location or @builtin(position)");
            int comps = t.k == Ty::Vec ? t.n : 1;
            if (t.scal() != Ty::F32 && t.scal() != Ty::I32 && t.scal() != Ty::U32)
                unsupported(vf->line, "inter-stage values of this type");
            const int it = interp_of(attrs, vf->line, t.scal() != Ty::F32);
            // integer values are carried bit for bit and must be flat (naga validates this; the
            // reference panics on anything else, fragment.rs:337-339)
            if (t.scal() != Ty::F32 && it != 2) bad(vf->line, "integer inter-stage values need @interpolate(flat)");
            slots.push_back(Slot{loc, comps, it});
            slot_kind_[loc] = t.scal();
            post_src_.push_back({loc, src, comps, t.k == Ty::Vec, t.scal()});
        };
        if (ret_ty_.k == Ty::Struct) {
            const StructDef* sd = structs_[ret_ty_.sid].first;
            const auto& mts = struct_member_types_[ret_ty_.sid];
            for (size_t i = 0; i < sd->members.size(); ++i) output(sd->members[i].attrs, mts[i], "o_.m_" + sd->members[i].name);
        } else {
            output(vf->ret_attrs, ret_ty_, "o_");
        }
        if (!have_pos) bad(vf->line, "vertex entry point does not write @builtin(position)");
        std::sort(slots.begin(), slots.end(), [](const Slot& a, const Slot& b) { return a.loc < b.loc; });
        std::sort(post_src_.begin(), post_src_.end(), [](const auto& a, const auto& b) { return std::get<0>(a) < std::get<0>(b); });
        int off = 0;
        for (size_t i = 0; i < post_src_.size(); ++i) {
            if (i && std::get<0>(post_src_[i]) == std::get<0>(post_src_[i - 1])) bad(vf->line, "duplicate output location");
            const auto& [loc, src, comps, isvec, sk] = post_src_[i];
            slot_off_[loc] = {off, comps};
            const char* conv = sk == Ty::I32 ? "__int_as_float" : sk == Ty::U32 ? "__uint_as_float" : "";
            for (int k = 0; k < comps; ++k)
                post << "  var[" << off + k << "] = " << conv << "(" << (isvec ? src + ".c[" + std::to_string(k) + "]" : src)
                     << ");\n";
            off += comps;
        }
        pc_.num_varyings = off;
        if (off > 16) unsupported(vf->line, "more than 16 inter-stage floats");
        // a vertex-only program: the interpolation its outputs declare (a fragment stage decides
        // below, from its inputs, as the reference does)
        if (!fs_) set_interpolation(slots, vf->line);
        std::ostringstream lam;
        stmts(vf->body, lam, 2);
        vw << "__device__ bool jit_vs(const DrawDesc& d, uint32_t vertex, uint32_t instance, V4& pos, float* var, uint32_t* err) {\n"
           << "  JitCtx __c{};\n  __c.d = &d;\n  (void)__c;\n  bool __tr = false;\n"
           << vinit.str() << decls.str() << pre.str()
           << "  const " << ctype(ret_ty_) << " o_ = [&]() -> " << ctype(ret_ty_) << " {\n" << lam.str()
           << "    return " << ctype(ret_ty_) << "{};\n  }();\n"
           << "  if (__tr) { *err = ERR_SHADER_TRAP; return false; }\n" << post.str() << "  return true;\n}\n";
    }

    // ---------- fragment stage
    std::ostringstream fw;
    std::ostringstream fmembers, finit;
    if (fs_) {
        mod_ = fs_;
        prefix_ = fs_ == &vs_ ? "v_" : "f_";
        const Func* ff = nullptr;
        for (const Func& f : fs_->funcs)
            if (f.name == fs_entry && f.stage == 1) ff = &f;
        if (!ff) throw Error("no @fragment entry point '" + fs_entry + "'", false);
        if (fs_ != &vs_) {
            emit_consts(*fs_, fconsts_);
            ctx_members(*fs_, fmembers, finit);
        }
        stage_ = 1;
        in_entry_ = true;
        scopes_.clear();
        push_globals(*fs_);
        push();
        std::ostringstream pre, decls;
        std::vector<Slot> fs_slots;  // the inputs at @location, with their interpolation
        // @early_depth_test(force) / @early_depth_test(<conservative depth>) (naga::EarlyDepthTest,
        // read by the reference at fragment.rs:83-86)
        for (const Attr& a : ff->attrs)
            if (a.name == "early_depth_test") {
                if (a.args.size() != 1) bad(ff->line, "@early_depth_test takes one argument");
                if (a.args[0] == "force") pc_.early_depth = 1;
                else if (a.args[0] == "greater_equal" || a.args[0] == "less_equal" || a.args[0] == "unchanged")
                    pc_.early_depth = 2;
                else bad(ff->line, "unknown @early_depth_test argument '" + a.args[0] + "'");
            }
        auto input = [&](const Member& p, const Ty& t, const std::string& dst) {
            std::string bname;
            if (builtin_of(p.attrs, &bname)) {
                if (bname == "position") {
                    if (t != Ty::vec(Ty::F32, 4)) bad(ff->line, "position must be vec4f");
                    pre << "  " << dst << " = WV<float,4>{frag.x, frag.y, frag.z, frag.w};\n";
                    pc_.uses_position = true;
                } else if (bname == "front_facing") {
                    pre << "  " << dst << " = front_facing;\n";
                } else if (bname == "primitive_index") {
                    pre << "  " << dst << " = prim_index;\n";
                } else if (bname == "sample_index") {
                    pre << "  " << dst << " = 0u;\n";
                } else if (bname == "sample_mask") {
                    pre << "  " << dst << " = 0xFFFFFFFFu;\n";
                } else {
                    unsupported(ff->line, "fragment input builtin " + bname);
                }
                return;
            }
            const int loc = location_of(p.attrs);
            auto it = slot_off_.find(loc);
            if (loc < 0 || it == slot_off_.end()) bad(ff->line, "fragment input @location(" + std::to_string(loc) + ") is not written by the vertex stage");
            const int comps = t.k == Ty::Vec ? t.n : 1;
            if (t.scal() != slot_kind_.at(loc) || comps != it->second.second)
                bad(ff->line, "fragment input type differs from the vertex output");
            // the fragment input's @interpolate decides how the value is interpolated
            // (Interpolation::from_naga on the input's binding, fragment.rs:250-262)
            const int interp = interp_of(p.attrs, ff->line, t.scal() != Ty::F32);
            if (t.scal() != Ty::F32 && interp != 2) bad(ff->line, "integer inter-stage values need @interpolate(flat)");
            fs_slots.push_back({loc, comps, interp});
            const char* conv = t.scal() == Ty::I32 ? "__float_as_int" : t.scal() == Ty::U32 ? "__float_as_uint" : "";
            for (int k = 0; k < comps; ++k)
                pre << "  " << (t.k == Ty::Vec ? dst + ".c[" + std::to_string(k) + "]" : dst) << " = " << conv << "(var["
                    << it->second.first + k << "]);\n";
        };
        for (const Member& p : ff->params) {
            Ty t = resolve(p.ty);
            const std::string c = declare(p.name, t, false, ff->line);
            decls << "  " << ctype(t) << " " << c << "{};\n";
            if (t.k == Ty::Struct) {
                const StructDef* sd = structs_[t.sid].first;
                const auto& mts = struct_member_types_[t.sid];
                for (size_t i = 0; i < sd->members.size(); ++i) input(sd->members[i], mts[i], c + ".m_" + sd->members[i].name);
            } else {
                input(p, t, c);
            }
        }
        // interpolation of the values the fragment stage reads: flat ones per float, one mode for
        // the others
        set_interpolation(fs_slots, ff->line);
        if (!ff->has_ret) unsupported(ff->line, "fragment entry point without a colour output");
        ret_ty_ = resolve(ff->ret);
        std::string colour;
        auto output = [&](const std::vector<Attr>& attrs, const Ty& t, const std::string& src) {
            std::string bname;
            if (builtin_of(attrs, &bname)) unsupported(ff->line, "fragment output builtin " + bname);
            const int loc = location_of(attrs);
            if (loc != 0) unsupported(ff->line, "colour outputs other than @location(0)");
            if (t != Ty::vec(Ty::F32, 4)) unsupported(ff->line, "a colour output that is not vec4f");
            colour = src;
        };
        if (ret_ty_.k == Ty::Struct) {
            const StructDef* sd = structs_[ret_ty_.sid].first;
            const auto& mts = struct_member_types_[ret_ty_.sid];
            for (size_t i = 0; i < sd->members.size(); ++i) output(sd->members[i].attrs, mts[i], "o_.m_" + sd->members[i].name);
        } else {
            output(ff->ret_attrs, ret_ty_, "o_");
        }
        if (colour.empty()) unsupported(ff->line, "fragment entry point without @location(0)");
        std::ostringstream lam;
        stmts(ff->body, lam, 2);
        fw << "// 0 = discarded, 1 = colour written, 2 = trap\n"
           << "__device__ int jit_fs(const DrawDesc& d, const float* var, bool front_facing, uint32_t prim_index, V4 frag, V4& color) {\n"
           << "  JitCtx __c{};\n  __c.d = &d;\n  (void)__c;\n  bool __tr = false;\n"
           << vinit.str() << finit.str() << decls.str() << pre.str()
           << "  const " << ctype(ret_ty_) << " o_ = [&]() -> " << ctype(ret_ty_) << " {\n" << lam.str()
           << "    return " << ctype(ret_ty_) << "{};\n  }();\n"
           << "  if (__tr) return 2;\n  if (__c.kill) return 0;\n"
           << "  color = V4{" << colour << ".c[0], " << colour << ".c[1], " << colour << ".c[2], " << colour << ".c[3]};\n"
           << "  return 1;\n}\n";
    }

    if (!fs_)  // a vertex-only program: the raster kernels still reference a fragment stage
        fw << "__device__ int jit_fs(const DrawDesc&, const float*, bool, uint32_t, V4, V4&) { return 0; }\n";
    // types, loaders and constants; the context; helper functions (which take it); the stages
    std::ostringstream out;
    out << decl_.str() << "struct JitCtx {\n  const DrawDesc* d;\n  bool kill;\n" << vmembers.str() << fmembers.str()
        << "};\n" << fns_.str() << vw.str() << fw.str();
    pc_.cuda = out.str();
    return pc_;
}

}  // namespace wgsl
}  // namespace gbr

namespace gbr {
namespace wgsl {
ProgramCode emit_program(const Module& vs, const std::string& vs_entry, const Module* fs, const std::string& fs_entry,
                         const Constants& vertex_constants, const Constants& fragment_constants) {
    // one module for both stages, with different constants per stage: the fragment stage gets a
    // copy of its own (its constants and globals are then emitted apart from the vertex stage's)
    Module fs_copy;
    if (fs == &vs && vertex_constants != fragment_constants) {
        fs_copy = vs;
        fs = &fs_copy;
    }
    Emitter em(vs, fs, vertex_constants, fragment_constants);
    return em.run(vs_entry, fs_entry);
}
}  // namespace wgsl
}  // namespace gbr
