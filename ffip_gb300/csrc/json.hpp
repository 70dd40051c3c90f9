// Small JSON reader for the simulation config (the schema ffip's Python
// front-end emits, ffip/simulation.py:362-402, and Simulation::init reads,
// src/simulation.cpp:127-188).  Values are immutable after parsing.
#pragma once
#include <cctype>
#include <cstdlib>
#include <map>
#include <memory>
#include <stdexcept>
#include <string>
#include <vector>

namespace ffipg
{
class Json
{
public:
    enum Kind { Null, Bool, Number, String, Array, Object };

    static Json parse(const std::string &text)
    {
        size_t p = 0;
        Json j = value(text, p);
        ws(text, p);
        if (p != text.size()) throw std::runtime_error("json: trailing characters at offset " + std::to_string(p));
        return j;
    }

    Kind kind() const { return k_; }
    bool is_null() const { return k_ == Null; }
    bool is_array() const { return k_ == Array; }
    bool is_object() const { return k_ == Object; }
    bool has(const std::string &key) const { return k_ == Object && obj_.count(key) != 0; }

    const Json &at(const std::string &key) const
    {
        if (k_ != Object) throw std::runtime_error("json: expected an object when reading key '" + key + "'");
        auto it = obj_.find(key);
        if (it == obj_.end()) throw std::runtime_error("json: missing key '" + key + "'");
        return it->second;
    }
    const Json &at(size_t i) const
    {
        if (k_ != Array || i >= arr_.size()) throw std::runtime_error("json: array index out of range");
        return arr_[i];
    }
    size_t size() const { return k_ == Array ? arr_.size() : 0; }
    const std::vector<Json> &items() const
    {
        static const std::vector<Json> empty;
        return k_ == Array ? arr_ : empty;
    }

    double num() const
    {
        if (k_ == Number) return num_;
        if (k_ == Bool) return b_ ? 1.0 : 0.0;
        throw std::runtime_error("json: expected a number");
    }
    int integer() const { return (int)num(); }
    const std::string &str() const
    {
        if (k_ != String) throw std::runtime_error("json: expected a string");
        return str_;
    }

    double num(const std::string &key, double dflt) const { return has(key) ? at(key).num() : dflt; }
    std::string str(const std::string &key, const std::string &dflt) const { return has(key) ? at(key).str() : dflt; }

private:
    Kind k_{Null};
    bool b_{false};
    double num_{0};
    std::string str_;
    std::vector<Json> arr_;
    std::map<std::string, Json> obj_;

    static void ws(const std::string &s, size_t &p)
    {
        while (p < s.size() && std::isspace((unsigned char)s[p])) ++p;
    }
    static void expect(const std::string &s, size_t &p, char c)
    {
        ws(s, p);
        if (p >= s.size() || s[p] != c) throw std::runtime_error(std::string("json: expected '") + c + "' at offset " + std::to_string(p));
        ++p;
    }
    static std::string string_lit(const std::string &s, size_t &p)
    {
        expect(s, p, '"');
        std::string out;
        while (p < s.size() && s[p] != '"')
        {
            char c = s[p++];
            if (c != '\\')
            {
                out += c;
                continue;
            }
            if (p >= s.size()) break;
            char e = s[p++];
            switch (e)
            {
            case 'n': out += '\n'; break;
            case 't': out += '\t'; break;
            case 'r': out += '\r'; break;
            case 'b': out += '\b'; break;
            case 'f': out += '\f'; break;
            case 'u':
            {
                unsigned cp = (unsigned)std::strtoul(s.substr(p, 4).c_str(), nullptr, 16);
                p += 4;
                if (cp < 0x80) out += (char)cp;
                else if (cp < 0x800) { out += (char)(0xC0 | (cp >> 6)); out += (char)(0x80 | (cp & 0x3F)); }
                else { out += (char)(0xE0 | (cp >> 12)); out += (char)(0x80 | ((cp >> 6) & 0x3F)); out += (char)(0x80 | (cp & 0x3F)); }
                break;
            }
            default: out += e;
            }
        }
        if (p >= s.size()) throw std::runtime_error("json: unterminated string");
        ++p;
        return out;
    }
    static Json value(const std::string &s, size_t &p)
    {
        ws(s, p);
        if (p >= s.size()) throw std::runtime_error("json: unexpected end of input");
        Json j;
        char c = s[p];
        if (c == '{')
        {
            j.k_ = Object;
            ++p;
            ws(s, p);
            if (p < s.size() && s[p] == '}') { ++p; return j; }
            for (;;)
            {
                std::string key = string_lit(s, p);
                expect(s, p, ':');
                j.obj_[key] = value(s, p);
                ws(s, p);
                if (p < s.size() && s[p] == ',') { ++p; continue; }
                expect(s, p, '}');
                break;
            }
        }
        else if (c == '[')
        {
            j.k_ = Array;
            ++p;
            ws(s, p);
            if (p < s.size() && s[p] == ']') { ++p; return j; }
            for (;;)
            {
                j.arr_.push_back(value(s, p));
                ws(s, p);
                if (p < s.size() && s[p] == ',') { ++p; continue; }
                expect(s, p, ']');
                break;
            }
        }
        else if (c == '"')
        {
            j.k_ = String;
            j.str_ = string_lit(s, p);
        }
        else if (s.compare(p, 4, "true") == 0) { j.k_ = Bool; j.b_ = true; p += 4; }
        else if (s.compare(p, 5, "false") == 0) { j.k_ = Bool; j.b_ = false; p += 5; }
        else if (s.compare(p, 4, "null") == 0) { p += 4; }
        else if (s.compare(p, 3, "NaN") == 0) { j.k_ = Number; j.num_ = std::strtod("nan", nullptr); p += 3; }
        else
        {
            const char *b = s.c_str() + p;
            char *e = nullptr;
            j.k_ = Number;
            j.num_ = std::strtod(b, &e);
            if (e == b) throw std::runtime_error("json: bad value at offset " + std::to_string(p));
            p += (size_t)(e - b);
        }
        return j;
    }
};
} // namespace ffipg
