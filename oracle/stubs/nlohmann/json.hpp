// Minimal stand-in for nlohmann::json (not installed in this build
// environment).  Test infrastructure only: enough of the API for the polysolve
// Solver interface and the adapter header (include/lss_polysolve.hpp) --
// parse, dump, operator[], assignment from scalars, key/value iteration over
// objects.  Numbers keep their source text, so values pass through unchanged.
#pragma once

#include <cctype>
#include <cstdio>
#include <map>
#include <stdexcept>
#include <string>
#include <utility>
#include <vector>

namespace nlohmann {

class json {
public:
    enum class kind { null, boolean, number, string, object, array };
    using member = std::pair<std::string, json>;

    json() = default;
    json(std::nullptr_t) {}
    json(bool b) : k_(kind::boolean), text_(b ? "true" : "false") {}
    json(int v) : k_(kind::number), text_(std::to_string(v)) {}
    json(long v) : k_(kind::number), text_(std::to_string(v)) {}
    json(long long v) : k_(kind::number), text_(std::to_string(v)) {}
    json(double v) : k_(kind::number)
    {
        char buf[40];
        std::snprintf(buf, sizeof buf, "%.17g", v);
        text_ = buf;
    }
    json(const char *s) : k_(kind::string), text_(s) {}
    json(const std::string &s) : k_(kind::string), text_(s) {}

    static json object() { json j; j.k_ = kind::object; return j; }

    static json parse(const char *s)
    {
        const char *p = s;
        json j = parse_value(p);
        skip(p);
        if (*p) throw std::runtime_error("json: trailing characters");
        return j;
    }
    static json parse(const std::string &s) { return parse(s.c_str()); }

    std::string dump() const
    {
        switch (k_) {
        case kind::null: return "null";
        case kind::boolean:
        case kind::number: return text_;
        case kind::string: return quote(text_);
        case kind::array: {
            std::string o = "[";
            for (size_t i = 0; i < arr_.size(); ++i) o += (i ? "," : "") + arr_[i].dump();
            return o + "]";
        }
        default: {
            std::string o = "{";
            for (size_t i = 0; i < obj_.size(); ++i)
                o += (i ? "," : "") + quote(obj_[i].first) + ":" + obj_[i].second.dump();
            return o + "}";
        }
        }
    }

    bool contains(const std::string &key) const
    {
        for (const auto &m : obj_)
            if (m.first == key) return true;
        return false;
    }
    json &operator[](const std::string &key)
    {
        if (k_ == kind::null) k_ = kind::object;
        for (auto &m : obj_)
            if (m.first == key) return m.second;
        obj_.emplace_back(key, json());
        return obj_.back().second;
    }
    json &operator[](const char *key) { return (*this)[std::string(key)]; }
    kind type() const { return k_; }
    const std::string &text() const { return text_; }
    double number() const { return std::stod(text_); }

    class iterator {
    public:
        iterator(std::vector<member> *v, size_t i) : v_(v), i_(i) {}
        bool operator!=(const iterator &o) const { return i_ != o.i_; }
        bool operator==(const iterator &o) const { return i_ == o.i_; }
        iterator &operator++()
        {
            ++i_;
            return *this;
        }
        const std::string &key() const { return (*v_)[i_].first; }
        json &value() const { return (*v_)[i_].second; }

    private:
        std::vector<member> *v_;
        size_t i_;
    };
    iterator begin() const { return iterator(const_cast<std::vector<member> *>(&obj_), 0); }
    iterator end() const { return iterator(const_cast<std::vector<member> *>(&obj_), obj_.size()); }

private:
    kind k_ = kind::null;
    std::string text_;
    std::vector<member> obj_;
    std::vector<json> arr_;

    static std::string quote(const std::string &s)
    {
        std::string o = "\"";
        for (char c : s) {
            if (c == '"' || c == '\\') o += '\\';
            o += c;
        }
        return o + "\"";
    }
    static void skip(const char *&p)
    {
        while (*p && std::isspace((unsigned char)*p)) ++p;
    }
    static std::string parse_string(const char *&p)
    {
        std::string s;
        ++p;  // opening quote
        while (*p && *p != '"') {
            if (*p == '\\' && p[1]) ++p;
            s += *p++;
        }
        if (*p != '"') throw std::runtime_error("json: unterminated string");
        ++p;
        return s;
    }
    static json parse_value(const char *&p)
    {
        skip(p);
        json j;
        if (*p == '{') {
            j.k_ = kind::object;
            ++p;
            skip(p);
            if (*p == '}') { ++p; return j; }
            for (;;) {
                skip(p);
                if (*p != '"') throw std::runtime_error("json: expected a key");
                std::string key = parse_string(p);
                skip(p);
                if (*p != ':') throw std::runtime_error("json: expected ':'");
                ++p;
                j.obj_.emplace_back(key, parse_value(p));
                skip(p);
                if (*p == ',') { ++p; continue; }
                if (*p == '}') { ++p; return j; }
                throw std::runtime_error("json: expected ',' or '}'");
            }
        }
        if (*p == '[') {
            j.k_ = kind::array;
            ++p;
            skip(p);
            if (*p == ']') { ++p; return j; }
            for (;;) {
                j.arr_.push_back(parse_value(p));
                skip(p);
                if (*p == ',') { ++p; continue; }
                if (*p == ']') { ++p; return j; }
                throw std::runtime_error("json: expected ',' or ']'");
            }
        }
        if (*p == '"') return json(parse_string(p));
        const char *q = p;
        while (*p && *p != ',' && *p != '}' && *p != ']' && !std::isspace((unsigned char)*p)) ++p;
        const std::string t(q, p);
        if (t == "null") return json();
        if (t == "true") return json(true);
        if (t == "false") return json(false);
        if (t.empty()) throw std::runtime_error("json: empty value");
        j.k_ = kind::number;
        j.text_ = t;
        return j;
    }
};

}  // namespace nlohmann
