// Minimal JSON value with the subset of the nlohmann::json interface that the
// reference's simulation driver uses (src/simulation.cpp, app/run_sim_json.cpp).
//
// Test infrastructure only: it lets the reference's own setup code parse a
// config.json when the reference is compiled here as the oracle.  Supported:
// parse from an istream, find/at/operator[] on objects, at(i) on arrays,
// begin()/end() iteration over array elements (or object values), get<T>() and
// get_to() for double/int/bool/std::string, and implicit conversion to double
// (used by `double_arr(j.begin(), j.end())`).
#pragma once
#include <cctype>
#include <cstdlib>
#include <istream>
#include <iterator>
#include <map>
#include <memory>
#include <stdexcept>
#include <string>
#include <utility>
#include <vector>

namespace nlohmann
{
class json
{
public:
    enum class kind { null, boolean, number, string, array, object };

    json() = default;
    json(double v) : k_(kind::number), num_(v) {}
    json(const std::string &s) : k_(kind::string), str_(s) {}

    // iterator over array elements, or over object values in key order
    template <typename J, typename VecIt, typename MapIt>
    struct iter_base
    {
        using iterator_category = std::forward_iterator_tag;
        using value_type = json;
        using difference_type = std::ptrdiff_t;
        using pointer = J *;
        using reference = J &;
        bool is_obj{false};
        VecIt vi{};
        MapIt mi{};
        J &operator*() const { return is_obj ? mi->second : *vi; }
        J *operator->() const { return &operator*(); }
        iter_base &operator++()
        {
            if (is_obj) ++mi;
            else ++vi;
            return *this;
        }
        iter_base operator++(int)
        {
            iter_base t = *this;
            ++*this;
            return t;
        }
        bool operator==(const iter_base &o) const { return is_obj ? mi == o.mi : vi == o.vi; }
        bool operator!=(const iter_base &o) const { return !(*this == o); }
    };
    using iterator = iter_base<json, std::vector<json>::iterator, std::map<std::string, json>::iterator>;
    using const_iterator = iter_base<const json, std::vector<json>::const_iterator, std::map<std::string, json>::const_iterator>;

    iterator begin()
    {
        iterator it;
        it.is_obj = (k_ == kind::object);
        if (it.is_obj) it.mi = obj_.begin();
        else it.vi = arr_.begin();
        return it;
    }
    iterator end()
    {
        iterator it;
        it.is_obj = (k_ == kind::object);
        if (it.is_obj) it.mi = obj_.end();
        else it.vi = arr_.end();
        return it;
    }
    const_iterator begin() const
    {
        const_iterator it;
        it.is_obj = (k_ == kind::object);
        if (it.is_obj) it.mi = obj_.cbegin();
        else it.vi = arr_.cbegin();
        return it;
    }
    const_iterator end() const
    {
        const_iterator it;
        it.is_obj = (k_ == kind::object);
        if (it.is_obj) it.mi = obj_.cend();
        else it.vi = arr_.cend();
        return it;
    }

    iterator find(const std::string &key)
    {
        if (k_ != kind::object) return end();
        iterator it;
        it.is_obj = true;
        it.mi = obj_.find(key);
        return it;
    }
    const_iterator find(const std::string &key) const
    {
        if (k_ != kind::object) return end();
        const_iterator it;
        it.is_obj = true;
        it.mi = obj_.find(key);
        return it;
    }

    const json &at(const std::string &key) const
    {
        if (k_ != kind::object) throw std::out_of_range("json: not an object, key " + key);
        auto it = obj_.find(key);
        if (it == obj_.end()) throw std::out_of_range("json: key not found: " + key);
        return it->second;
    }
    json &at(const std::string &key) { return const_cast<json &>(static_cast<const json &>(*this).at(key)); }
    const json &at(size_t i) const
    {
        if (k_ != kind::array || i >= arr_.size()) throw std::out_of_range("json: bad array index");
        return arr_[i];
    }
    json &at(size_t i) { return const_cast<json &>(static_cast<const json &>(*this).at(i)); }
    const json &at(int i) const { return at((size_t)i); }
    json &at(int i) { return at((size_t)i); }

    const json &operator[](const std::string &key) const { return at(key); }
    json &operator[](const std::string &key)
    {
        if (k_ == kind::null) k_ = kind::object;
        return obj_[key];
    }
    const json &operator[](const char *key) const { return at(std::string(key)); }
    json &operator[](const char *key) { return operator[](std::string(key)); }

    size_t size() const { return k_ == kind::array ? arr_.size() : k_ == kind::object ? obj_.size() : (k_ == kind::null ? 0 : 1); }
    bool is_null() const { return k_ == kind::null; }

    template <typename T>
    T get() const
    {
        T v;
        get_to(v);
        return v;
    }
    void get_to(double &v) const { v = as_number(); }
    void get_to(float &v) const { v = (float)as_number(); }
    void get_to(int &v) const { v = (int)as_number(); }
    void get_to(long &v) const { v = (long)as_number(); }
    void get_to(unsigned &v) const { v = (unsigned)as_number(); }
    void get_to(bool &v) const
    {
        if (k_ == kind::boolean) v = bool_;
        else v = as_number() != 0;
    }
    void get_to(std::string &v) const
    {
        if (k_ != kind::string) throw std::runtime_error("json: not a string");
        v = str_;
    }
    operator double() const { return as_number(); }

    friend std::istream &operator>>(std::istream &is, json &j)
    {
        std::string text((std::istreambuf_iterator<char>(is)), std::istreambuf_iterator<char>());
        size_t pos = 0;
        j = parse_value(text, pos);
        return is;
    }

private:
    kind k_{kind::null};
    bool bool_{false};
    double num_{0};
    std::string str_;
    std::vector<json> arr_;
    std::map<std::string, json> obj_;

    double as_number() const
    {
        if (k_ == kind::number) return num_;
        if (k_ == kind::boolean) return bool_ ? 1.0 : 0.0;
        throw std::runtime_error("json: not a number");
    }

    static void skip_ws(const std::string &s, size_t &p)
    {
        while (p < s.size() && std::isspace((unsigned char)s[p])) ++p;
    }
    static std::string parse_string(const std::string &s, size_t &p)
    {
        if (s[p] != '"') throw std::runtime_error("json: expected string");
        ++p;
        std::string out;
        while (p < s.size() && s[p] != '"')
        {
            char c = s[p++];
            if (c == '\\')
            {
                char e = s[p++];
                switch (e)
                {
                case 'n': out += '\n'; break;
                case 't': out += '\t'; break;
                case 'r': out += '\r'; break;
                case 'b': out += '\b'; break;
                case 'f': out += '\f'; break;
                case 'u': out += '?'; p += 4; break;
                default: out += e;
                }
            }
            else
                out += c;
        }
        ++p;
        return out;
    }
    static json parse_value(const std::string &s, size_t &p)
    {
        skip_ws(s, p);
        if (p >= s.size()) throw std::runtime_error("json: unexpected end");
        json j;
        char c = s[p];
        if (c == '{')
        {
            j.k_ = kind::object;
            ++p;
            skip_ws(s, p);
            if (s[p] == '}') { ++p; return j; }
            while (true)
            {
                skip_ws(s, p);
                std::string key = parse_string(s, p);
                skip_ws(s, p);
                if (s[p] != ':') throw std::runtime_error("json: expected ':'");
                ++p;
                j.obj_[key] = parse_value(s, p);
                skip_ws(s, p);
                if (s[p] == ',') { ++p; continue; }
                if (s[p] == '}') { ++p; break; }
                throw std::runtime_error("json: expected ',' or '}'");
            }
        }
        else if (c == '[')
        {
            j.k_ = kind::array;
            ++p;
            skip_ws(s, p);
            if (s[p] == ']') { ++p; return j; }
            while (true)
            {
                j.arr_.push_back(parse_value(s, p));
                skip_ws(s, p);
                if (s[p] == ',') { ++p; continue; }
                if (s[p] == ']') { ++p; break; }
                throw std::runtime_error("json: expected ',' or ']'");
            }
        }
        else if (c == '"')
        {
            j.k_ = kind::string;
            j.str_ = parse_string(s, p);
        }
        else if (s.compare(p, 4, "true") == 0) { j.k_ = kind::boolean; j.bool_ = true; p += 4; }
        else if (s.compare(p, 5, "false") == 0) { j.k_ = kind::boolean; j.bool_ = false; p += 5; }
        else if (s.compare(p, 4, "null") == 0) { p += 4; }
        else
        {
            const char *b = s.c_str() + p;
            char *e = nullptr;
            j.k_ = kind::number;
            j.num_ = std::strtod(b, &e);
            if (e == b) throw std::runtime_error("json: bad number");
            p += (size_t)(e - b);
        }
        return j;
    }
};
} // namespace nlohmann
