// Test-infrastructure shim (oracle build only; never linked into the product).
//
// A small JSON value type named nlohmann::json that supplies exactly the API
// subset the reference's src/utils/json.cpp:1-209 calls, so that the
// reference's own hot-path headers compile here without the third-party
// nlohmann/json library (not vendored, src/utils/json.hpp:3, .gitignore:2).
// Written from scratch for this project; it is not nlohmann source.
//
// Behaviour mirrored from the library call the reference makes,
// parse(input, nullptr, /*allow_exceptions=*/true, /*ignore_comments=*/true):
//   * // line and /* block */ comments are skipped as whitespace;
//   * numbers without '.', 'e' or 'E' are integers (negative -> int64,
//     non-negative -> uint64, too large -> double); others are doubles
//     converted with strtod (correctly rounded on glibc);
//   * a duplicate object key keeps the last value;
//   * trailing non-whitespace after the root value is an error;
//   * errors throw std::runtime_error.
#pragma once

#include <algorithm>
#include <cerrno>
#include <cmath>
#include <cstdint>
#include <cstdlib>
#include <cstring>
#include <functional>
#include <iostream>
#include <iterator>
#include <map>
#include <memory>
#include <sstream>
#include <stdexcept>
#include <string>
#include <type_traits>
#include <unordered_map>
#include <vector>

namespace nlohmann
{

class json
{
public:
    enum class kind { null, boolean, integer, unsigned_int, floating, string,
        array, object };
    using array_t = std::vector<json>;
    using object_t = std::map<std::string, json>;

    // opaque iterator for find()/end() comparisons
    struct const_iterator
    {
        const json *owner = nullptr;
        bool at_end = true;
        object_t::const_iterator it;
        bool operator==(const const_iterator& o) const
        {
            if (at_end || o.at_end)
                return at_end == o.at_end;
            return it == o.it;
        }
        bool operator!=(const const_iterator& o) const { return !(*this == o); }
    };

private:
    kind k_ = kind::null;
    bool b_ = false;
    int64_t i_ = 0;
    uint64_t u_ = 0;
    double d_ = 0.0;
    std::string s_;
    std::shared_ptr<array_t> a_;
    std::shared_ptr<object_t> o_;

    struct reader
    {
        const std::string& t;
        size_t p = 0;
        explicit reader(const std::string& text): t(text) {}

        [[noreturn]] void fail(const std::string& why) const
        {
            throw std::runtime_error("json parse error at byte "
                + std::to_string(p) + ": " + why);
        }

        void skip()
        {
            for (;;)
            {
                while (p < t.size() && (t[p] == ' ' || t[p] == '\t'
                        || t[p] == '\n' || t[p] == '\r'))
                    ++p;
                if (p + 1 < t.size() && t[p] == '/' && t[p+1] == '/')
                {
                    p += 2;
                    while (p < t.size() && t[p] != '\n')
                        ++p;
                    continue;
                }
                if (p + 1 < t.size() && t[p] == '/' && t[p+1] == '*')
                {
                    size_t e = t.find("*/", p + 2);
                    if (e == std::string::npos)
                        fail("unterminated comment");
                    p = e + 2;
                    continue;
                }
                if (p < t.size() && t[p] == '/')
                    fail("invalid comment");
                return;
            }
        }

        static void put_utf8(std::string& out, uint32_t cp)
        {
            if (cp < 0x80)
                out += (char)cp;
            else if (cp < 0x800)
            {
                out += (char)(0xC0 | (cp >> 6));
                out += (char)(0x80 | (cp & 0x3F));
            }
            else if (cp < 0x10000)
            {
                out += (char)(0xE0 | (cp >> 12));
                out += (char)(0x80 | ((cp >> 6) & 0x3F));
                out += (char)(0x80 | (cp & 0x3F));
            }
            else
            {
                out += (char)(0xF0 | (cp >> 18));
                out += (char)(0x80 | ((cp >> 12) & 0x3F));
                out += (char)(0x80 | ((cp >> 6) & 0x3F));
                out += (char)(0x80 | (cp & 0x3F));
            }
        }

        uint32_t hex4()
        {
            if (p + 4 > t.size())
                fail("short \\u escape");
            uint32_t v = 0;
            for (int j = 0; j < 4; ++j)
            {
                char c = t[p++];
                v <<= 4;
                if (c >= '0' && c <= '9') v |= (uint32_t)(c - '0');
                else if (c >= 'a' && c <= 'f') v |= (uint32_t)(c - 'a' + 10);
                else if (c >= 'A' && c <= 'F') v |= (uint32_t)(c - 'A' + 10);
                else fail("bad hex digit");
            }
            return v;
        }

        std::string str()
        {
            if (t[p] != '"')
                fail("expected string");
            ++p;
            std::string out;
            for (;;)
            {
                if (p >= t.size())
                    fail("unterminated string");
                unsigned char c = (unsigned char)t[p++];
                if (c == '"')
                    return out;
                if (c < 0x20)
                    fail("control character in string");
                if (c != '\\')
                {
                    out += (char)c;
                    continue;
                }
                if (p >= t.size())
                    fail("bad escape");
                char e = t[p++];
                switch (e)
                {
                case '"': out += '"'; break;
                case '\\': out += '\\'; break;
                case '/': out += '/'; break;
                case 'b': out += '\b'; break;
                case 'f': out += '\f'; break;
                case 'n': out += '\n'; break;
                case 'r': out += '\r'; break;
                case 't': out += '\t'; break;
                case 'u':
                {
                    uint32_t cp = hex4();
                    if (cp >= 0xD800 && cp <= 0xDBFF)
                    {
                        if (p + 2 > t.size() || t[p] != '\\' || t[p+1] != 'u')
                            fail("lone surrogate");
                        p += 2;
                        uint32_t lo = hex4();
                        if (lo < 0xDC00 || lo > 0xDFFF)
                            fail("bad surrogate pair");
                        cp = 0x10000 + ((cp - 0xD800) << 10) + (lo - 0xDC00);
                    }
                    else if (cp >= 0xDC00 && cp <= 0xDFFF)
                        fail("lone surrogate");
                    put_utf8(out, cp);
                    break;
                }
                default: fail("bad escape");
                }
            }
        }

        json number()
        {
            size_t s = p;
            bool neg = false, isfloat = false;
            if (t[p] == '-') { neg = true; ++p; }
            if (p >= t.size() || !(t[p] >= '0' && t[p] <= '9'))
                fail("bad number");
            if (t[p] == '0')
                ++p;
            else
                while (p < t.size() && t[p] >= '0' && t[p] <= '9') ++p;
            if (p < t.size() && t[p] == '.')
            {
                isfloat = true;
                ++p;
                if (p >= t.size() || !(t[p] >= '0' && t[p] <= '9'))
                    fail("bad fraction");
                while (p < t.size() && t[p] >= '0' && t[p] <= '9') ++p;
            }
            if (p < t.size() && (t[p] == 'e' || t[p] == 'E'))
            {
                isfloat = true;
                ++p;
                if (p < t.size() && (t[p] == '+' || t[p] == '-')) ++p;
                if (p >= t.size() || !(t[p] >= '0' && t[p] <= '9'))
                    fail("bad exponent");
                while (p < t.size() && t[p] >= '0' && t[p] <= '9') ++p;
            }
            std::string tok = t.substr(s, p - s);
            json j;
            if (!isfloat)
            {
                errno = 0;
                if (neg)
                {
                    long long v = std::strtoll(tok.c_str(), nullptr, 10);
                    if (errno == 0)
                    {
                        j.k_ = kind::integer;
                        j.i_ = v;
                        return j;
                    }
                }
                else
                {
                    unsigned long long v = std::strtoull(tok.c_str(), nullptr, 10);
                    if (errno == 0)
                    {
                        j.k_ = kind::unsigned_int;
                        j.u_ = v;
                        return j;
                    }
                }
            }
            j.k_ = kind::floating;
            j.d_ = std::strtod(tok.c_str(), nullptr);
            if (!std::isfinite(j.d_))
                fail("number out of range");
            return j;
        }

        json value(int depth)
        {
            if (depth > 512)
                fail("nesting too deep");
            skip();
            if (p >= t.size())
                fail("unexpected end of input");
            char c = t[p];
            json j;
            if (c == '{')
            {
                ++p;
                j.k_ = kind::object;
                j.o_ = std::make_shared<object_t>();
                skip();
                if (p < t.size() && t[p] == '}') { ++p; return j; }
                for (;;)
                {
                    skip();
                    if (p >= t.size()) fail("unexpected end in object");
                    std::string key = str();
                    skip();
                    if (p >= t.size() || t[p] != ':') fail("expected ':'");
                    ++p;
                    (*j.o_)[key] = value(depth + 1);
                    skip();
                    if (p < t.size() && t[p] == ',') { ++p; continue; }
                    if (p < t.size() && t[p] == '}') { ++p; return j; }
                    fail("expected ',' or '}'");
                }
            }
            if (c == '[')
            {
                ++p;
                j.k_ = kind::array;
                j.a_ = std::make_shared<array_t>();
                skip();
                if (p < t.size() && t[p] == ']') { ++p; return j; }
                for (;;)
                {
                    j.a_->push_back(value(depth + 1));
                    skip();
                    if (p < t.size() && t[p] == ',') { ++p; continue; }
                    if (p < t.size() && t[p] == ']') { ++p; return j; }
                    fail("expected ',' or ']'");
                }
            }
            if (c == '"')
            {
                j.k_ = kind::string;
                j.s_ = str();
                return j;
            }
            if (t.compare(p, 4, "true") == 0) { p += 4; j.k_ = kind::boolean; j.b_ = true; return j; }
            if (t.compare(p, 5, "false") == 0) { p += 5; j.k_ = kind::boolean; j.b_ = false; return j; }
            if (t.compare(p, 4, "null") == 0) { p += 4; return j; }
            if (c == '-' || (c >= '0' && c <= '9'))
                return number();
            fail("unexpected character");
        }
    };

    static void dump_string(std::ostream& os, const std::string& s)
    {
        os << '"';
        for (unsigned char c : s)
        {
            switch (c)
            {
            case '"': os << "\\\""; break;
            case '\\': os << "\\\\"; break;
            case '\n': os << "\\n"; break;
            case '\r': os << "\\r"; break;
            case '\t': os << "\\t"; break;
            default:
                if (c < 0x20)
                {
                    char buf[8];
                    std::snprintf(buf, sizeof buf, "\\u%04x", c);
                    os << buf;
                }
                else
                    os << (char)c;
            }
        }
        os << '"';
    }

public:
    json() = default;
    json(const json&) = default;
    json& operator=(const json&) = default;

    static json parse(const std::string& text, std::nullptr_t = nullptr,
        bool allow_exceptions = true, bool ignore_comments = true)
    {
        (void)allow_exceptions;
        (void)ignore_comments;
        reader r(text);
        json j = r.value(0);
        r.skip();
        if (r.p != text.size())
            r.fail("trailing characters");
        return j;
    }

    static json parse(std::istream& in, std::nullptr_t = nullptr,
        bool allow_exceptions = true, bool ignore_comments = true)
    {
        std::string text((std::istreambuf_iterator<char>(in)),
            std::istreambuf_iterator<char>());
        return parse(text, nullptr, allow_exceptions, ignore_comments);
    }

    bool is_null() const noexcept { return k_ == kind::null; }
    bool is_boolean() const noexcept { return k_ == kind::boolean; }
    bool is_number_integer() const noexcept
    { return k_ == kind::integer || k_ == kind::unsigned_int; }
    bool is_number() const noexcept
    { return is_number_integer() || k_ == kind::floating; }
    bool is_string() const noexcept { return k_ == kind::string; }
    bool is_array() const noexcept { return k_ == kind::array; }
    bool is_object() const noexcept { return k_ == kind::object; }

    size_t size() const noexcept
    {
        if (k_ == kind::array) return a_->size();
        if (k_ == kind::object) return o_->size();
        if (k_ == kind::null) return 0;
        return 1;
    }

    template <typename T>
    T get() const
    {
        if constexpr (std::is_same_v<T, bool>)
        {
            if (k_ != kind::boolean) throw std::runtime_error("type must be boolean");
            return b_;
        }
        else if constexpr (std::is_same_v<T, std::string>)
        {
            if (k_ != kind::string) throw std::runtime_error("type must be string");
            return s_;
        }
        else if constexpr (std::is_same_v<T, std::vector<json>>)
        {
            if (k_ != kind::array) throw std::runtime_error("type must be array");
            return *a_;
        }
        else if constexpr (std::is_same_v<T, std::unordered_map<std::string, json>>)
        {
            if (k_ != kind::object) throw std::runtime_error("type must be object");
            return T(o_->begin(), o_->end());
        }
        else if constexpr (std::is_arithmetic_v<T>)
        {
            switch (k_)
            {
            case kind::integer: return static_cast<T>(i_);
            case kind::unsigned_int: return static_cast<T>(u_);
            case kind::floating: return static_cast<T>(d_);
            case kind::boolean: throw std::runtime_error("type must be number");
            default: throw std::runtime_error("type must be number");
            }
        }
        else
            static_assert(sizeof(T) == 0, "unsupported get<T>");
    }

    const json& at(size_t i) const
    {
        if (k_ != kind::array) throw std::runtime_error("at(): not an array");
        if (i >= a_->size()) throw std::runtime_error("at(): index out of range");
        return (*a_)[i];
    }

    const json& at(const std::string& key) const
    {
        if (k_ != kind::object) throw std::runtime_error("at(): not an object");
        auto it = o_->find(key);
        if (it == o_->end()) throw std::runtime_error("at(): key not found");
        return it->second;
    }

    const_iterator find(const std::string& key) const
    {
        const_iterator r;
        r.owner = this;
        if (k_ != kind::object)
            return r;
        auto it = o_->find(key);
        if (it == o_->end())
            return r;
        r.at_end = false;
        r.it = it;
        return r;
    }

    const_iterator end() const
    {
        const_iterator r;
        r.owner = this;
        return r;
    }

    bool operator==(const json& o) const
    {
        if (is_number() && o.is_number())
        {
            if (k_ == kind::floating || o.k_ == kind::floating)
                return get<double>() == o.get<double>();
            if (k_ == o.k_)
                return k_ == kind::integer ? i_ == o.i_ : u_ == o.u_;
            int64_t si = k_ == kind::integer ? i_ : o.i_;
            uint64_t uu = k_ == kind::unsigned_int ? u_ : o.u_;
            return si >= 0 && (uint64_t)si == uu;
        }
        if (k_ != o.k_) return false;
        switch (k_)
        {
        case kind::null: return true;
        case kind::boolean: return b_ == o.b_;
        case kind::string: return s_ == o.s_;
        case kind::array: return *a_ == *o.a_;
        case kind::object: return *o_ == *o.o_;
        default: return false;
        }
    }

    friend std::ostream& operator<<(std::ostream& os, const json& j)
    {
        switch (j.k_)
        {
        case kind::null: os << "null"; break;
        case kind::boolean: os << (j.b_ ? "true" : "false"); break;
        case kind::integer: os << j.i_; break;
        case kind::unsigned_int: os << j.u_; break;
        case kind::floating:
        {
            char buf[32];
            std::snprintf(buf, sizeof buf, "%.17g", j.d_);
            os << buf;
            break;
        }
        case kind::string: dump_string(os, j.s_); break;
        case kind::array:
        {
            os << '[';
            bool first = true;
            for (const json& e : *j.a_)
            {
                if (!first) os << ',';
                first = false;
                os << e;
            }
            os << ']';
            break;
        }
        case kind::object:
        {
            os << '{';
            bool first = true;
            for (const auto& kv : *j.o_)
            {
                if (!first) os << ',';
                first = false;
                dump_string(os, kv.first);
                os << ':' << kv.second;
            }
            os << '}';
            break;
        }
        }
        return os;
    }
};

} // namespace nlohmann
