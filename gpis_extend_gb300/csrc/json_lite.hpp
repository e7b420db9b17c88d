// json_lite.hpp -- a small JSON reader for medium descriptions (scene-JSON
// subset: objects, arrays, numbers, strings, booleans, null).
#pragma once

#include <cstdlib>
#include <map>
#include <memory>
#include <stdexcept>
#include <string>
#include <vector>

namespace gpis {
namespace json {

struct Value {
    enum Kind { Null, Bool, Number, String, Array, Object } kind = Null;
    bool b = false;
    double num = 0.0;
    std::string str;
    std::vector<Value> arr;
    std::map<std::string, Value> obj;

    const Value *get(const std::string &key) const {
        if (kind != Object) return nullptr;
        auto it = obj.find(key);
        return it == obj.end() ? nullptr : &it->second;
    }
};

class Parser {
    const char *p_;
    const char *end_;

    [[noreturn]] void fail(const char *what) {
        throw std::runtime_error(std::string("JSON parse error: ") + what);
    }
    void ws() {
        while (p_ < end_ && (*p_ == ' ' || *p_ == '\n' || *p_ == '\r' || *p_ == '\t')) ++p_;
    }
    bool lit(const char *s) {
        const char *q = p_;
        while (*s) {
            if (q >= end_ || *q != *s) return false;
            ++q; ++s;
        }
        p_ = q;
        return true;
    }
    std::string string_body() {
        if (p_ >= end_ || *p_ != '"') fail("expected string");
        ++p_;
        std::string out;
        while (p_ < end_ && *p_ != '"') {
            char c = *p_++;
            if (c == '\\') {
                if (p_ >= end_) fail("bad escape");
                char e = *p_++;
                switch (e) {
                case 'n': out += '\n'; break;
                case 't': out += '\t'; break;
                case 'r': out += '\r'; break;
                case 'b': out += '\b'; break;
                case 'f': out += '\f'; break;
                case 'u': {
                    if (end_ - p_ < 4) fail("bad unicode escape");
                    unsigned cp = (unsigned)std::strtoul(std::string(p_, 4).c_str(), nullptr, 16);
                    p_ += 4;
                    if (cp < 0x80) out += (char)cp;
                    else out += '?';
                    break;
                }
                default: out += e;
                }
            } else {
                out += c;
            }
        }
        if (p_ >= end_) fail("unterminated string");
        ++p_;
        return out;
    }
    Value value() {
        ws();
        if (p_ >= end_) fail("unexpected end");
        Value v;
        const char c = *p_;
        if (c == '{') {
            ++p_;
            v.kind = Value::Object;
            ws();
            if (p_ < end_ && *p_ == '}') { ++p_; return v; }
            for (;;) {
                ws();
                std::string k = string_body();
                ws();
                if (p_ >= end_ || *p_ != ':') fail("expected ':'");
                ++p_;
                v.obj[k] = value();
                ws();
                if (p_ < end_ && *p_ == ',') { ++p_; continue; }
                if (p_ < end_ && *p_ == '}') { ++p_; break; }
                fail("expected ',' or '}'");
            }
        } else if (c == '[') {
            ++p_;
            v.kind = Value::Array;
            ws();
            if (p_ < end_ && *p_ == ']') { ++p_; return v; }
            for (;;) {
                v.arr.push_back(value());
                ws();
                if (p_ < end_ && *p_ == ',') { ++p_; continue; }
                if (p_ < end_ && *p_ == ']') { ++p_; break; }
                fail("expected ',' or ']'");
            }
        } else if (c == '"') {
            v.kind = Value::String;
            v.str = string_body();
        } else if (lit("true")) {
            v.kind = Value::Bool; v.b = true;
        } else if (lit("false")) {
            v.kind = Value::Bool; v.b = false;
        } else if (lit("null")) {
            v.kind = Value::Null;
        } else {
            char *q = nullptr;
            v.num = std::strtod(p_, &q);
            if (q == p_) fail("bad token");
            v.kind = Value::Number;
            p_ = q;
        }
        return v;
    }

public:
    explicit Parser(const std::string &s) : p_(s.data()), end_(s.data() + s.size()) {}
    Value parse() {
        Value v = value();
        ws();
        if (p_ != end_) fail("trailing characters");
        return v;
    }
};

inline Value parse(const std::string &s) { return Parser(s).parse(); }

}  // namespace json
}  // namespace gpis
