// pt_glsl.cpp — GLSL SDF snippets to C++ over pt_glsl_shim.h.
//
// The reference splices a scene's `sdf[i].glsl` text into its compute shader
// and recompiles it (src/pathtracer.cpp:2004-2054, InsertSDF).  Here the text
// is rewritten into C++ that the shim header gives GLSL meaning to, then
// compiled for the GPU at run time (pt_jit.cu) and, in the tests, for the CPU
// restatement.  The rewrite works on tokens:
//   - comments are dropped;
//   - float literals get an f suffix (GLSL floats are single precision);
//   - read swizzles (.xz, .zyx, .rg ...) become member calls (.xz()), and
//     single rgba components name the fields (.g -> .y);
//   - assignment to a swizzle of a variable, `v.xy = e;` or `v.xy op= e;`,
//     becomes `v.set_xy(e);` or `v.set_xy(v.xy() op (e));`;
//   - a vector constructor with two or more arguments that call a snippet
//     function with out/inout parameters, `vec2(rnd(seed), rnd(seed))`, is
//     braced (`vec2{...}`): GLSL evaluates arguments left to right, C++
//     only guarantees that order in a braced list;
//   - parameter qualifiers: `in`/`const in` are dropped, `out`/`inout` make
//     the parameter a reference;
//   - every function the snippet defines is renamed <prefix><name> and
//     marked as a device function, and the whole text goes into namespace
//     ptg::<prefix>, so several snippets (or one in several slots) coexist;
//   - top-level `const float|int` declarations become constexpr.
//   - struct declarations pass through (C++ reads them the same way), and
//     their names count as types from then on.
// Anything the shim does not cover (uniforms, preprocessor lines, arrays of
// vectors at file scope...) is rejected with a message instead of being
// guessed at.
#include <cctype>
#include <cstring>
#include <set>
#include <string>
#include <vector>

#include "../../include/pt_cuda.h"

namespace {

struct Tok {
    enum Kind { Ident, Number, Punct, Space } kind;
    std::string text;
};

bool is_swizzle(const std::string& s) {
    if (s.size() < 2 || s.size() > 4) return false;
    const bool xyzw = s.find_first_not_of("xyzw") == std::string::npos;
    const bool rgba = s.find_first_not_of("rgba") == std::string::npos;
    return xyzw || rgba;
}

std::string rgba_to_xyzw(std::string s) {
    for (char& c : s) {
        if (c == 'r') c = 'x';
        else if (c == 'g') c = 'y';
        else if (c == 'b') c = 'z';
        else if (c == 'a') c = 'w';
    }
    return s;
}

bool is_type(const std::string& s) {
    static const std::set<std::string> types = {"float", "int",   "uint",  "bool",  "void",  "vec2",  "vec3", "vec4",
                                                "mat2",  "mat3",  "uvec2", "ivec2", "bvec2", "bvec3", "bvec4"};
    return types.count(s) != 0;
}

// Splits the text into tokens, dropping comments.  Returns false on an
// unterminated comment.
bool tokenize(const std::string& src, std::vector<Tok>& out, std::string& err) {
    size_t i = 0;
    const size_t n = src.size();
    while (i < n) {
        const char c = src[i];
        if (c == '/' && i + 1 < n && src[i + 1] == '/') {
            while (i < n && src[i] != '\n') i++;
            continue;
        }
        if (c == '/' && i + 1 < n && src[i + 1] == '*') {
            const size_t e = src.find("*/", i + 2);
            if (e == std::string::npos) {
                err = "unterminated comment";
                return false;
            }
            i = e + 2;
            out.push_back({Tok::Space, " "});
            continue;
        }
        if (std::isspace((unsigned char)c)) {
            size_t j = i;
            while (j < n && std::isspace((unsigned char)src[j])) j++;
            out.push_back({Tok::Space, src.substr(i, j - i)});
            i = j;
            continue;
        }
        if (std::isalpha((unsigned char)c) || c == '_') {
            size_t j = i;
            while (j < n && (std::isalnum((unsigned char)src[j]) || src[j] == '_')) j++;
            out.push_back({Tok::Ident, src.substr(i, j - i)});
            i = j;
            continue;
        }
        const bool leading_dot = (c == '.' && i + 1 < n && std::isdigit((unsigned char)src[i + 1]) &&
                                  (out.empty() || (out.back().kind != Tok::Ident && out.back().text != ")" &&
                                                   out.back().text != "]")));
        if (std::isdigit((unsigned char)c) || leading_dot) {
            size_t j = i;
            while (j < n && (std::isalnum((unsigned char)src[j]) || src[j] == '.' ||
                             ((src[j] == '+' || src[j] == '-') && (src[j - 1] == 'e' || src[j - 1] == 'E'))))
                j++;
            out.push_back({Tok::Number, src.substr(i, j - i)});
            i = j;
            continue;
        }
        out.push_back({Tok::Punct, std::string(1, c)});
        i++;
    }
    return true;
}

// The literal as a C++ float (or int) literal.
std::string float_literal(const std::string& t) {
    std::string s = t;
    if (!s.empty() && (s.back() == 'f' || s.back() == 'F')) s.pop_back();
    const bool is_float = s.find_first_of(".eE") != std::string::npos && s.compare(0, 2, "0x") != 0;
    if (!is_float) return s;
    if (s.back() == '.') s += "0";
    if (s.front() == '.') s = "0" + s;
    return s + "f";
}

size_t next_nonspace(const std::vector<Tok>& t, size_t i) {
    while (i < t.size() && t[i].kind == Tok::Space) i++;
    return i;
}

}  // namespace

extern "C" int pt_glsl_translate(const char* glsl, const char* prefix, char* out, size_t cap, size_t* needed,
                                 char* err, size_t err_cap) {
    auto fail = [&](const std::string& m) {
        if (err && err_cap) {
            std::strncpy(err, m.c_str(), err_cap - 1);
            err[err_cap - 1] = '\0';
        }
        return PT_ERR_UNSUPPORTED;
    };
    if (!glsl || !prefix) return PT_ERR_INVALID;
    // the prefix names a namespace and starts function names: an identifier
    if (!(std::isalpha((unsigned char)prefix[0]) || prefix[0] == '_')) return fail("the prefix must be an identifier");
    for (const char* c = prefix; *c; c++)
        if (!(std::isalnum((unsigned char)*c) || *c == '_')) return fail("the prefix must be an identifier");
    std::vector<Tok> t;
    std::string e;
    if (!tokenize(glsl, t, e)) return fail(e);

    // Struct types the snippet declares (`struct Name {` at file scope), and
    // their member names (a member called r, g, b or a keeps its name).
    std::set<std::string> structs, members;
    for (size_t i = 0; i < t.size(); i++)
        if (t[i].kind == Tok::Ident && t[i].text == "struct") {
            const size_t j = next_nonspace(t, i + 1);
            if (j >= t.size() || t[j].kind != Tok::Ident) return fail("a struct needs a name");
            structs.insert(t[j].text);
            size_t q = next_nonspace(t, j + 1);
            if (q >= t.size() || t[q].text != "{") return fail("a struct needs a body");
            for (size_t prev = q; q < t.size() && t[q].text != "}"; q++) {
                if (t[q].kind == Tok::Space) continue;
                if ((t[q].text == ";" || t[q].text == ",") && t[prev].kind == Tok::Ident)
                    members.insert(t[prev].text);  // `float a, b;` declares both
                prev = q;
            }
        }
    auto type_like = [&](const std::string& w) { return is_type(w) || structs.count(w) != 0; };

    // Functions the snippet defines: `type name (` at brace depth 0, and
    // those of them with out/inout parameters (calls with side effects).
    std::set<std::string> funcs, effect_funcs;
    int depth = 0;
    for (size_t i = 0; i < t.size(); i++) {
        if (t[i].kind == Tok::Punct) {
            if (t[i].text == "{") depth++;
            if (t[i].text == "}") depth--;
            if (t[i].text == "#") return fail("preprocessor lines are not supported");
            continue;
        }
        if (t[i].kind != Tok::Ident) continue;
        if (t[i].text == "uniform" || t[i].text == "layout" || t[i].text == "buffer")
            return fail("'" + t[i].text + "' is not supported in an SDF snippet");
        if (depth == 0 && type_like(t[i].text)) {
            const size_t j = next_nonspace(t, i + 1);
            const size_t k = j < t.size() ? next_nonspace(t, j + 1) : t.size();
            if (j < t.size() && t[j].kind == Tok::Ident && k < t.size() && t[k].text == "(") {
                funcs.insert(t[j].text);
                for (size_t q = k + 1; q < t.size() && t[q].text != ")"; q++)
                    if (t[q].text == "out" || t[q].text == "inout") effect_funcs.insert(t[j].text);
            }
        }
    }
    if (!funcs.count("sdf") || !funcs.count("sdfmaterial"))
        return fail("the snippet must define float sdf(vec3) and float sdfmaterial(vec3)");

    // Each snippet in its own namespace, so that file-scope constants of two
    // snippets (or of one snippet in two slots) do not collide.
    std::string o = "namespace ptg {\nnamespace " + std::string(prefix) + " {\n";
    depth = 0;
    int paren = 0;
    bool ref_pending = false;  // out/inout seen: the next type gets '&'
    std::string close_stmt;    // closes a rewritten swizzle assignment at its ';'
    std::set<size_t> brace_close;  // ')' tokens of braced constructors
    for (size_t i = 0; i < t.size(); i++) {
        const Tok& k = t[i];
        if (k.kind == Tok::Space) {
            o += k.text;
            continue;
        }
        if (!close_stmt.empty() && k.kind == Tok::Punct && paren == 0 && (k.text == ";" || k.text == "," ||
                                                                          k.text == "{" || k.text == "}")) {
            if (k.text != ";") return fail("a swizzle assignment must be a statement of its own");
            o += close_stmt;
            close_stmt.clear();
        }
        if (k.kind == Tok::Number) {
            o += float_literal(k.text);
            continue;
        }
        if (k.kind == Tok::Punct) {
            if (k.text == "{") depth++;
            if (k.text == "}") depth--;
            if (k.text == "(") paren++;
            if (k.text == ")") paren--;
            if (k.text == ")" && brace_close.count(i)) {
                o += "}";
                continue;
            }
            if (k.text == ".") {
                const size_t j = i + 1;  // swizzles follow the dot directly
                if (j < t.size() && t[j].kind == Tok::Ident && is_swizzle(t[j].text)) {
                    const std::string sw = rgba_to_xyzw(t[j].text);
                    const size_t a = next_nonspace(t, j + 1);
                    // `=` or `op=` (the tokenizer gives single-character punctuation)
                    std::string op;
                    size_t eq = t.size();
                    if (a < t.size() && t[a].text == "=" && !(a + 1 < t.size() && t[a + 1].text == "=")) {
                        eq = a;
                    } else if (a + 1 < t.size() && (t[a].text == "+" || t[a].text == "-" || t[a].text == "*" ||
                                                     t[a].text == "/") &&
                               t[a + 1].text == "=" && !(a + 2 < t.size() && t[a + 2].text == "=")) {
                        op = t[a].text;
                        eq = a + 1;
                    }
                    if (eq < t.size()) {
                        // the target: a plain variable, written just before the dot
                        size_t b = i;
                        while (b > 0 && t[b - 1].kind == Tok::Space) b--;
                        if (b == 0 || t[b - 1].kind != Tok::Ident || !close_stmt.empty())
                            return fail("assignment to a swizzle needs a plain variable on the left");
                        size_t bb = b - 1;
                        while (bb > 0 && t[bb - 1].kind == Tok::Space) bb--;
                        if (bb > 0 && (t[bb - 1].text == "." || t[bb - 1].text == "]" || t[bb - 1].text == ")"))
                            return fail("assignment to a swizzle needs a plain variable on the left");
                        const std::string var = t[b - 1].text;
                        o += ".set_" + sw + "(";
                        if (!op.empty()) o += var + "." + sw + "() " + op + " (";
                        close_stmt = op.empty() ? ")" : "))";
                        i = eq;
                        continue;
                    }
                    o += "." + sw + "()";
                    i = j;
                    continue;
                }
                // single components: .r .g .b .a name the fields x y z w
                // (unless a struct of the snippet has a member of that name)
                if (j < t.size() && t[j].kind == Tok::Ident && t[j].text.size() == 1 &&
                    std::strchr("rgba", t[j].text[0]) && !members.count(t[j].text)) {
                    o += "." + rgba_to_xyzw(t[j].text);
                    i = j;
                    continue;
                }
            }
            o += k.text;
            continue;
        }
        // identifiers
        const std::string& w = k.text;
        if (w == "in" || w == "highp" || w == "mediump" || w == "lowp") continue;
        if (w == "out" || w == "inout") {
            ref_pending = true;
            continue;
        }
        if (w == "const" && depth == 0 && paren == 0) {
            const size_t j = next_nonspace(t, i + 1);
            if (j < t.size() && (t[j].text == "float" || t[j].text == "int")) {
                o += "constexpr";
                continue;
            }
            return fail("file-scope constants must be float or int");
        }
        if (depth == 0 && paren == 0 && type_like(w)) {
            const size_t j = next_nonspace(t, i + 1);
            const size_t n2 = j < t.size() ? next_nonspace(t, j + 1) : t.size();
            if (j < t.size() && t[j].kind == Tok::Ident && funcs.count(t[j].text) && n2 < t.size() && t[n2].text == "(")
                o += "PTG_FN ";
        }
        if (funcs.count(w)) {
            o += std::string(prefix) + w;
            if (ref_pending && type_like(w)) {  // a struct that shares a function's name
                o += "&";
                ref_pending = false;
            }
            continue;
        }
        if (type_like(w) && w != "void" && !effect_funcs.empty()) {
            // a constructor call: count its arguments that call a function with side effects
            const size_t open = next_nonspace(t, i + 1);
            if (open < t.size() && t[open].text == "(") {
                int d = 0, effects = 0;
                bool arg_effect = false;
                size_t close = open;
                for (size_t q = open; q < t.size(); q++) {
                    const std::string& x = t[q].text;
                    if (x == "(") d++;
                    if (x == ")" && --d == 0) {
                        close = q;
                        break;
                    }
                    if (d == 1 && x == ",") {
                        effects += arg_effect;
                        arg_effect = false;
                    }
                    if (t[q].kind == Tok::Ident && effect_funcs.count(x)) arg_effect = true;
                }
                effects += arg_effect;
                if (close > open && effects >= 2) {
                    o += w + "{";
                    paren++;
                    brace_close.insert(close);
                    i = open;
                    continue;
                }
            }
        }
        o += w;
        if (ref_pending && type_like(w)) {
            o += "&";
            ref_pending = false;
        }
    }
    if (depth != 0 || paren != 0) return fail("unbalanced braces or parentheses");
    o += "\n}  // namespace " + std::string(prefix) + "\n}  // namespace ptg\n";
    if (needed) *needed = o.size() + 1;
    if (!out) return PT_OK;
    if (cap < o.size() + 1) return PT_ERR_INVALID;
    std::memcpy(out, o.c_str(), o.size() + 1);
    return PT_OK;
}
