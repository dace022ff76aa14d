// pt_json.cpp — recursive-descent JSON parser and printer (RFC 8259 subset
// that scene files use: no duplicate-key semantics beyond "last wins").
#include "pt_json.h"

#include <cerrno>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>

namespace ptjson {

const Value* Value::find(const std::string& key) const {
    if (type != Object) return nullptr;
    for (auto it = obj.rbegin(); it != obj.rend(); ++it)
        if (it->first == key) return &it->second;
    return nullptr;
}

Value& Value::at_or_insert(const std::string& key) {
    if (type != Object) {
        *this = make_object();
    }
    for (auto& kv : obj)
        if (kv.first == key) return kv.second;
    obj.emplace_back(key, Value());
    return obj.back().second;
}

namespace {

struct Parser {
    const std::string& t;
    size_t p = 0;
    std::string err;
    int depth = 0;

    explicit Parser(const std::string& text) : t(text) {}

    bool fail(const char* msg) {
        if (err.empty()) err = std::string(msg) + " at byte " + std::to_string(p);
        return false;
    }
    void ws() {
        while (p < t.size() && (t[p] == ' ' || t[p] == '\t' || t[p] == '\n' || t[p] == '\r')) ++p;
    }
    bool lit(const char* s) {
        const size_t n = std::strlen(s);
        if (t.compare(p, n, s) != 0) return false;
        p += n;
        return true;
    }
    static void utf8(std::string& out, uint32_t cp) {
        if (cp < 0x80) {
            out += (char)cp;
        } else if (cp < 0x800) {
            out += (char)(0xC0 | (cp >> 6));
            out += (char)(0x80 | (cp & 0x3F));
        } else if (cp < 0x10000) {
            out += (char)(0xE0 | (cp >> 12));
            out += (char)(0x80 | ((cp >> 6) & 0x3F));
            out += (char)(0x80 | (cp & 0x3F));
        } else {
            out += (char)(0xF0 | (cp >> 18));
            out += (char)(0x80 | ((cp >> 12) & 0x3F));
            out += (char)(0x80 | ((cp >> 6) & 0x3F));
            out += (char)(0x80 | (cp & 0x3F));
        }
    }
    bool hex4(uint32_t& v) {
        if (p + 4 > t.size()) return fail("truncated \\u escape");
        v = 0;
        for (int i = 0; i < 4; i++) {
            const char c = t[p++];
            v <<= 4;
            if (c >= '0' && c <= '9') v |= (uint32_t)(c - '0');
            else if (c >= 'a' && c <= 'f') v |= (uint32_t)(c - 'a' + 10);
            else if (c >= 'A' && c <= 'F') v |= (uint32_t)(c - 'A' + 10);
            else return fail("bad hex digit in \\u escape");
        }
        return true;
    }
    bool string(std::string& out) {
        if (p >= t.size() || t[p] != '"') return fail("expected string");
        ++p;
        out.clear();
        while (p < t.size()) {
            const unsigned char c = (unsigned char)t[p++];
            if (c == '"') return true;
            if (c < 0x20) return fail("control character in string");
            if (c != '\\') {
                out += (char)c;
                continue;
            }
            if (p >= t.size()) break;
            const char e = t[p++];
            switch (e) {
                case '"': out += '"'; break;
                case '\\': out += '\\'; break;
                case '/': out += '/'; break;
                case 'b': out += '\b'; break;
                case 'f': out += '\f'; break;
                case 'n': out += '\n'; break;
                case 'r': out += '\r'; break;
                case 't': out += '\t'; break;
                case 'u': {
                    uint32_t cp = 0;
                    if (!hex4(cp)) return false;
                    if (cp >= 0xD800 && cp <= 0xDBFF) {
                        uint32_t lo = 0;
                        if (!lit("\\u") || !hex4(lo) || lo < 0xDC00 || lo > 0xDFFF) return fail("bad surrogate pair");
                        cp = 0x10000 + ((cp - 0xD800) << 10) + (lo - 0xDC00);
                    } else if (cp >= 0xDC00 && cp <= 0xDFFF) {
                        return fail("lone low surrogate");
                    }
                    utf8(out, cp);
                    break;
                }
                default: return fail("bad escape");
            }
        }
        return fail("unterminated string");
    }
    bool number(Value& v) {
        const size_t s = p;
        if (p < t.size() && t[p] == '-') ++p;
        if (p >= t.size() || !(t[p] >= '0' && t[p] <= '9')) return fail("bad number");
        if (t[p] == '0') {
            ++p;
        } else {
            while (p < t.size() && t[p] >= '0' && t[p] <= '9') ++p;
        }
        bool is_float = false;
        if (p < t.size() && t[p] == '.') {
            is_float = true;
            ++p;
            if (p >= t.size() || !(t[p] >= '0' && t[p] <= '9')) return fail("bad fraction");
            while (p < t.size() && t[p] >= '0' && t[p] <= '9') ++p;
        }
        if (p < t.size() && (t[p] == 'e' || t[p] == 'E')) {
            is_float = true;
            ++p;
            if (p < t.size() && (t[p] == '+' || t[p] == '-')) ++p;
            if (p >= t.size() || !(t[p] >= '0' && t[p] <= '9')) return fail("bad exponent");
            while (p < t.size() && t[p] >= '0' && t[p] <= '9') ++p;
        }
        const std::string tok = t.substr(s, p - s);
        if (!is_float) {
            errno = 0;
            char* end = nullptr;
            const long long iv = std::strtoll(tok.c_str(), &end, 10);
            if (errno == 0 && end && *end == '\0') {
                v = Value::make_int(iv);
                return true;
            }
        }
        v = Value::make_float(std::strtod(tok.c_str(), nullptr));
        return true;
    }
    bool value(Value& v) {
        if (++depth > 256) return fail("nesting too deep");
        ws();
        if (p >= t.size()) return fail("unexpected end");
        const char c = t[p];
        bool ok;
        if (c == '{') {
            ++p;
            v = Value::make_object();
            ws();
            if (p < t.size() && t[p] == '}') {
                ++p;
                ok = true;
            } else {
                ok = false;
                for (;;) {
                    ws();
                    std::string key;
                    if (!string(key)) break;
                    ws();
                    if (p >= t.size() || t[p] != ':') {
                        fail("expected ':'");
                        break;
                    }
                    ++p;
                    Value item;
                    if (!value(item)) break;
                    bool replaced = false;
                    for (auto& kv : v.obj)
                        if (kv.first == key) {
                            kv.second = std::move(item);
                            replaced = true;
                            break;
                        }
                    if (!replaced) v.obj.emplace_back(std::move(key), std::move(item));
                    ws();
                    if (p < t.size() && t[p] == ',') {
                        ++p;
                        continue;
                    }
                    if (p < t.size() && t[p] == '}') {
                        ++p;
                        ok = true;
                    } else {
                        fail("expected ',' or '}'");
                    }
                    break;
                }
            }
        } else if (c == '[') {
            ++p;
            v = Value::make_array();
            ws();
            if (p < t.size() && t[p] == ']') {
                ++p;
                ok = true;
            } else {
                ok = false;
                for (;;) {
                    Value item;
                    if (!value(item)) break;
                    v.arr.push_back(std::move(item));
                    ws();
                    if (p < t.size() && t[p] == ',') {
                        ++p;
                        continue;
                    }
                    if (p < t.size() && t[p] == ']') {
                        ++p;
                        ok = true;
                    } else {
                        fail("expected ',' or ']'");
                    }
                    break;
                }
            }
        } else if (c == '"') {
            v = Value::make_string("");
            ok = string(v.s);
        } else if (lit("true")) {
            v = Value::make_bool(true);
            ok = true;
        } else if (lit("false")) {
            v = Value::make_bool(false);
            ok = true;
        } else if (lit("null")) {
            v = Value();
            ok = true;
        } else {
            ok = number(v);
        }
        --depth;
        return ok;
    }
};

// Shortest decimal that reads back as the same double, laid out like common
// JSON writers: plain notation for decimal exponents in (-4, 15], otherwise
// d.ddde+XX; integral values keep a ".0" so floats stay floats.
std::string format_double(double d) {
    if (!std::isfinite(d)) return "null";
    if (d == 0.0) return std::signbit(d) ? "-0.0" : "0.0";
    char buf[48];
    int prec = 1;
    for (; prec <= 17; prec++) {
        std::snprintf(buf, sizeof buf, "%.*e", prec - 1, d);
        if (std::strtod(buf, nullptr) == d) break;
    }
    // buf = [-]d.ddde[+-]xx : split digits and exponent.
    std::string s(buf), sign;
    if (s[0] == '-') {
        sign = "-";
        s = s.substr(1);
    }
    const size_t epos = s.find('e');
    const int e10 = std::atoi(s.c_str() + epos + 1);
    std::string digits;
    for (size_t i = 0; i < epos; i++)
        if (s[i] != '.') digits += s[i];
    while (digits.size() > 1 && digits.back() == '0') digits.pop_back();
    const int k = (int)digits.size();
    const int n = e10 + 1;  // value = 0.digits * 10^n
    std::string out;
    if (k <= n && n <= 15) {
        out = digits + std::string((size_t)(n - k), '0') + ".0";
    } else if (0 < n && n <= 15) {
        out = digits.substr(0, (size_t)n) + "." + digits.substr((size_t)n);
    } else if (-4 < n && n <= 0) {
        out = "0." + std::string((size_t)(-n), '0') + digits;
    } else {
        char eb[16];
        std::snprintf(eb, sizeof eb, "e%c%02d", (n - 1) < 0 ? '-' : '+', std::abs(n - 1));
        out = digits.substr(0, 1) + (k > 1 ? "." + digits.substr(1) : std::string()) + eb;
    }
    return sign + out;
}

void escape(std::string& out, const std::string& s) {
    out += '"';
    size_t i = 0;
    while (i < s.size()) {
        const unsigned char c = (unsigned char)s[i];
        if (c == '"') out += "\\\"";
        else if (c == '\\') out += "\\\\";
        else if (c == '\b') out += "\\b";
        else if (c == '\f') out += "\\f";
        else if (c == '\n') out += "\\n";
        else if (c == '\r') out += "\\r";
        else if (c == '\t') out += "\\t";
        else if (c < 0x20 || c >= 0x80) {
            uint32_t cp = c;
            int extra = 0;
            if (c >= 0xF0) { cp = c & 0x07; extra = 3; }
            else if (c >= 0xE0) { cp = c & 0x0F; extra = 2; }
            else if (c >= 0xC0) { cp = c & 0x1F; extra = 1; }
            for (int k = 0; k < extra && i + 1 < s.size(); k++) cp = (cp << 6) | ((unsigned char)s[++i] & 0x3F);
            char buf[16];
            if (cp >= 0x10000) {
                cp -= 0x10000;
                std::snprintf(buf, sizeof buf, "\\u%04x\\u%04x", 0xD800 + (cp >> 10), 0xDC00 + (cp & 0x3FF));
            } else {
                std::snprintf(buf, sizeof buf, "\\u%04x", cp);
            }
            out += buf;
        } else {
            out += (char)c;
        }
        ++i;
    }
    out += '"';
}

void dump_rec(const Value& v, int indent, int level, std::string& out) {
    const std::string pad((size_t)(indent * (level + 1)), ' ');
    const std::string pad0((size_t)(indent * level), ' ');
    switch (v.type) {
        case Value::Null: out += "null"; break;
        case Value::Bool: out += v.b ? "true" : "false"; break;
        case Value::Int: out += std::to_string(v.i); break;
        case Value::Float: out += format_double(v.d); break;
        case Value::String: escape(out, v.s); break;
        case Value::Array:
            if (v.arr.empty()) {
                out += "[]";
                break;
            }
            out += "[\n";
            for (size_t k = 0; k < v.arr.size(); k++) {
                out += pad;
                dump_rec(v.arr[k], indent, level + 1, out);
                if (k + 1 < v.arr.size()) out += ',';
                out += '\n';
            }
            out += pad0 + "]";
            break;
        case Value::Object:
            if (v.obj.empty()) {
                out += "{}";
                break;
            }
            out += "{\n";
            for (size_t k = 0; k < v.obj.size(); k++) {
                out += pad;
                escape(out, v.obj[k].first);
                out += ": ";
                dump_rec(v.obj[k].second, indent, level + 1, out);
                if (k + 1 < v.obj.size()) out += ',';
                out += '\n';
            }
            out += pad0 + "}";
            break;
    }
}

}  // namespace

bool parse(const std::string& text, Value& out, std::string& err) {
    Parser ps(text);
    Value v;
    if (!ps.value(v)) {
        err = ps.err.empty() ? "parse error" : ps.err;
        return false;
    }
    ps.ws();
    if (ps.p != text.size()) {
        err = "trailing characters at byte " + std::to_string(ps.p);
        return false;
    }
    out = std::move(v);
    return true;
}

std::string dump(const Value& v, int indent) {
    std::string out;
    dump_rec(v, indent, 0, out);
    return out;
}

}  // namespace ptjson
