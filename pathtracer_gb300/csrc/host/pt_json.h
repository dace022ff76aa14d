// pt_json.h — a small JSON value, parser and pretty-printer for scene files.
//
// Objects keep insertion order (the reference reads and writes scenes with an
// order-preserving JSON object); numbers remember whether they were written
// as integers, so a scene round-trips through load and save.
#pragma once

#include <cstdint>
#include <string>
#include <utility>
#include <vector>

namespace ptjson {

struct Value {
    enum Type { Null, Bool, Int, Float, String, Array, Object };
    Type type = Null;
    bool b = false;
    int64_t i = 0;
    double d = 0.0;
    std::string s;
    std::vector<Value> arr;
    std::vector<std::pair<std::string, Value>> obj;

    static Value make_int(int64_t v) {
        Value x;
        x.type = Int;
        x.i = v;
        return x;
    }
    static Value make_float(double v) {
        Value x;
        x.type = Float;
        x.d = v;
        return x;
    }
    static Value make_bool(bool v) {
        Value x;
        x.type = Bool;
        x.b = v;
        return x;
    }
    static Value make_string(const std::string& v) {
        Value x;
        x.type = String;
        x.s = v;
        return x;
    }
    static Value make_array() {
        Value x;
        x.type = Array;
        return x;
    }
    static Value make_object() {
        Value x;
        x.type = Object;
        return x;
    }

    bool is_number() const { return type == Int || type == Float || type == Bool; }
    double number() const { return type == Int ? (double)i : (type == Bool ? (b ? 1.0 : 0.0) : d); }
    const Value* find(const std::string& key) const;
    // Object member access that inserts (like operator[] on a mutable object).
    Value& at_or_insert(const std::string& key);
};

// Parses `text`; on failure returns false and a message with the byte offset.
bool parse(const std::string& text, Value& out, std::string& err);

// Pretty-prints with `indent` spaces per level; non-ASCII escaped as \uXXXX.
std::string dump(const Value& v, int indent);

}  // namespace ptjson
