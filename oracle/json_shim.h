// A minimal stand-in for nlohmann::json with only the calls the
// reference's Nerfstudio and Polycam loaders make (core/src/loaders/
// load_nerfstudio.cpp, load_polycam.cpp), so those files compile unchanged
// here, where nlohmann's library is not installed — TEST INFRASTRUCTURE
// ONLY.  Semantics follow nlohmann's documentation for these calls: numbers
// without a fraction or exponent are integers, others doubles (strtod);
// get<T>() converts a number with static_cast; value(key, default) is the
// key's value converted to the default's type, or the default when the key
// is absent; operator[] on an object inserts null for a missing key;
// iterating an array yields its elements and an object its values in key
// order (nlohmann's default object is a std::map).
#pragma once

#include <cctype>
#include <cstdint>
#include <cstdlib>
#include <istream>
#include <iterator>
#include <stdexcept>
#include <string>
#include <type_traits>
#include <utility>
#include <vector>

namespace nlohmann {

class json {
public:
    enum class Kind { Null, Bool, Int, Float, String, Array, Object };

    static json parse(std::istream &in) {
        const std::string text((std::istreambuf_iterator<char>(in)), std::istreambuf_iterator<char>());
        size_t pos = 0;
        json j = parse_value(text, pos);
        skip_ws(text, pos);
        if (pos != text.size()) throw std::runtime_error("json: trailing characters");
        return j;
    }

    bool contains(const std::string &key) const { return kind_ == Kind::Object && find(key) >= 0; }

    json &operator[](const std::string &key) {
        if (kind_ == Kind::Null) kind_ = Kind::Object;
        if (kind_ != Kind::Object) throw std::runtime_error("json: not an object");
        const long i = find(key);
        if (i >= 0) return items_[(size_t)i];
        size_t at = 0;   // keep the keys sorted, as nlohmann's std::map does
        while (at < keys_.size() && keys_[at] < key) at++;
        keys_.insert(keys_.begin() + (long)at, key);
        return *items_.insert(items_.begin() + (long)at, json());
    }
    json &operator[](const char *key) { return (*this)[std::string(key)]; }
    json &operator[](size_t idx) {
        if (kind_ != Kind::Array || idx >= items_.size()) throw std::runtime_error("json: bad array index");
        return items_[idx];
    }
    json &operator[](int idx) { return (*this)[(size_t)idx]; }

    template <class T> T get() const {
        if constexpr (std::is_same_v<T, std::string>) {
            if (kind_ != Kind::String) throw std::runtime_error("json: not a string");
            return str_;
        } else if constexpr (std::is_same_v<T, bool>) {
            if (kind_ != Kind::Bool) throw std::runtime_error("json: not a boolean");
            return b_;
        } else {
            static_assert(std::is_arithmetic_v<T>, "json: numbers, strings and booleans only");
            if (kind_ == Kind::Int) return static_cast<T>(i_);
            if (kind_ == Kind::Float) return static_cast<T>(d_);
            throw std::runtime_error("json: not a number");
        }
    }

    template <class T> T value(const std::string &key, const T &fallback) const {
        const long i = kind_ == Kind::Object ? find(key) : -1;
        return i >= 0 ? items_[(size_t)i].get<T>() : fallback;
    }
    std::string value(const std::string &key, const char *fallback) const {
        return value<std::string>(key, std::string(fallback));
    }

    std::vector<json>::iterator begin() { return items_.begin(); }
    std::vector<json>::iterator end() { return items_.end(); }

private:
    Kind kind_ = Kind::Null;
    bool b_ = false;
    int64_t i_ = 0;
    double d_ = 0.0;
    std::string str_;
    std::vector<std::string> keys_;   // objects: sorted keys, values in items_
    std::vector<json> items_;         // array elements or object values

    long find(const std::string &key) const {
        for (size_t k = 0; k < keys_.size(); k++)
            if (keys_[k] == key) return (long)k;
        return -1;
    }

    static void skip_ws(const std::string &t, size_t &p) {
        while (p < t.size() && (t[p] == ' ' || t[p] == '\t' || t[p] == '\n' || t[p] == '\r')) p++;
    }
    static void expect(const std::string &t, size_t &p, const char *word) {
        for (const char *c = word; *c; c++, p++)
            if (p >= t.size() || t[p] != *c) throw std::runtime_error("json: bad literal");
    }
    static void put_utf8(std::string &out, unsigned cp) {
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
    static unsigned hex4(const std::string &t, size_t &p) {
        if (p + 4 > t.size()) throw std::runtime_error("json: bad escape");
        const unsigned v = (unsigned)std::stoul(t.substr(p, 4), nullptr, 16);
        p += 4;
        return v;
    }
    static std::string parse_string(const std::string &t, size_t &p) {
        std::string out;
        p++;   // opening quote
        while (p < t.size() && t[p] != '"') {
            char c = t[p++];
            if (c != '\\') {
                out += c;
                continue;
            }
            if (p >= t.size()) break;
            c = t[p++];
            switch (c) {
                case 'b': out += '\b'; break;
                case 'f': out += '\f'; break;
                case 'n': out += '\n'; break;
                case 'r': out += '\r'; break;
                case 't': out += '\t'; break;
                case 'u': {
                    unsigned cp = hex4(t, p);
                    if (cp >= 0xD800 && cp < 0xDC00 && p + 1 < t.size() && t[p] == '\\' && t[p + 1] == 'u') {
                        p += 2;
                        cp = 0x10000 + ((cp - 0xD800) << 10) + (hex4(t, p) - 0xDC00);
                    }
                    put_utf8(out, cp);
                    break;
                }
                default: out += c;   // \" \\ \/
            }
        }
        if (p >= t.size()) throw std::runtime_error("json: unterminated string");
        p++;   // closing quote
        return out;
    }
    static json parse_value(const std::string &t, size_t &p) {
        skip_ws(t, p);
        if (p >= t.size()) throw std::runtime_error("json: unexpected end");
        json j;
        const char c = t[p];
        if (c == '{') {
            j.kind_ = Kind::Object;
            p++;
            skip_ws(t, p);
            if (p < t.size() && t[p] == '}') { p++; return j; }
            while (true) {
                skip_ws(t, p);
                if (p >= t.size() || t[p] != '"') throw std::runtime_error("json: expected a key");
                const std::string key = parse_string(t, p);
                skip_ws(t, p);
                if (p >= t.size() || t[p] != ':') throw std::runtime_error("json: expected ':'");
                p++;
                j[key] = parse_value(t, p);
                skip_ws(t, p);
                if (p < t.size() && t[p] == ',') { p++; continue; }
                if (p < t.size() && t[p] == '}') { p++; return j; }
                throw std::runtime_error("json: expected ',' or '}'");
            }
        }
        if (c == '[') {
            j.kind_ = Kind::Array;
            p++;
            skip_ws(t, p);
            if (p < t.size() && t[p] == ']') { p++; return j; }
            while (true) {
                j.items_.push_back(parse_value(t, p));
                skip_ws(t, p);
                if (p < t.size() && t[p] == ',') { p++; continue; }
                if (p < t.size() && t[p] == ']') { p++; return j; }
                throw std::runtime_error("json: expected ',' or ']'");
            }
        }
        if (c == '"') {
            j.kind_ = Kind::String;
            j.str_ = parse_string(t, p);
            return j;
        }
        if (c == 't') { expect(t, p, "true"); j.kind_ = Kind::Bool; j.b_ = true; return j; }
        if (c == 'f') { expect(t, p, "false"); j.kind_ = Kind::Bool; j.b_ = false; return j; }
        if (c == 'n') { expect(t, p, "null"); return j; }
        // a number: an integer unless it has a fraction or an exponent
        const size_t start = p;
        bool is_float = false;
        while (p < t.size() && (std::isdigit((unsigned char)t[p]) || t[p] == '-' || t[p] == '+' || t[p] == '.' ||
                                t[p] == 'e' || t[p] == 'E')) {
            if (t[p] == '.' || t[p] == 'e' || t[p] == 'E') is_float = true;
            p++;
        }
        if (p == start) throw std::runtime_error("json: unexpected character");
        const std::string num = t.substr(start, p - start);
        if (is_float) {
            j.kind_ = Kind::Float;
            j.d_ = std::strtod(num.c_str(), nullptr);
        } else {
            j.kind_ = Kind::Int;
            j.i_ = std::strtoll(num.c_str(), nullptr, 10);
        }
        return j;
    }
};

}  // namespace nlohmann
