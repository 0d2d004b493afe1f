// JSON reader for flame files; behaviour documented in json.hpp.
#include "json.hpp"

#include <cerrno>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <sstream>

namespace ffr {

class JsonReader
{
public:
    explicit JsonReader(const std::string& t) : t_(t) {}

    JsonValue document()
    {
        JsonValue v = value(0);
        ws();
        if (pos_ != t_.size())
            fail("unexpected trailing characters");
        return v;
    }

private:
    const std::string& t_;
    size_t pos_ = 0;

    [[noreturn]] void fail(const std::string& why) const
    {
        // report a line number like a text editor would
        size_t line = 1;
        for (size_t k = 0; k < pos_ && k < t_.size(); ++k)
            line += t_[k] == '\n';
        throw FlameError("json parse error (line " + std::to_string(line)
            + "): " + why);
    }

    bool at_end() const { return pos_ >= t_.size(); }
    char peek() const { return t_[pos_]; }

    void ws()
    {
        while (!at_end())
        {
            char c = peek();
            if (c == ' ' || c == '\t' || c == '\n' || c == '\r')
            {
                ++pos_;
            }
            else if (c == '/' && pos_ + 1 < t_.size() && t_[pos_ + 1] == '/')
            {
                size_t e = t_.find('\n', pos_);
                pos_ = e == std::string::npos ? t_.size() : e;
            }
            else if (c == '/' && pos_ + 1 < t_.size() && t_[pos_ + 1] == '*')
            {
                size_t e = t_.find("*/", pos_ + 2);
                if (e == std::string::npos)
                    fail("unterminated block comment");
                pos_ = e + 2;
            }
            else
                return;
        }
    }

    void expect(char c)
    {
        if (at_end() || peek() != c)
            fail(std::string("expected '") + c + "'");
        ++pos_;
    }

    unsigned hex4()
    {
        if (pos_ + 4 > t_.size())
            fail("truncated \\u escape");
        unsigned v = 0;
        for (int k = 0; k < 4; ++k)
        {
            char c = t_[pos_++];
            v <<= 4;
            if (c >= '0' && c <= '9') v += (unsigned)(c - '0');
            else if (c >= 'a' && c <= 'f') v += (unsigned)(c - 'a' + 10);
            else if (c >= 'A' && c <= 'F') v += (unsigned)(c - 'A' + 10);
            else fail("invalid \\u escape");
        }
        return v;
    }

    static void utf8(std::string& o, unsigned cp)
    {
        if (cp < 0x80) { o += (char)cp; return; }
        if (cp < 0x800)
        {
            o += (char)(0xC0 | (cp >> 6));
        }
        else if (cp < 0x10000)
        {
            o += (char)(0xE0 | (cp >> 12));
            o += (char)(0x80 | ((cp >> 6) & 0x3F));
        }
        else
        {
            o += (char)(0xF0 | (cp >> 18));
            o += (char)(0x80 | ((cp >> 12) & 0x3F));
            o += (char)(0x80 | ((cp >> 6) & 0x3F));
        }
        o += (char)(0x80 | (cp & 0x3F));
    }

    std::string string_lit()
    {
        expect('"');
        std::string o;
        for (;;)
        {
            if (at_end())
                fail("unterminated string");
            unsigned char c = (unsigned char)t_[pos_++];
            if (c == '"')
                return o;
            if (c < 0x20)
                fail("control character in string");
            if (c != '\\')
            {
                o += (char)c;
                continue;
            }
            if (at_end())
                fail("unterminated escape");
            char e = t_[pos_++];
            switch (e)
            {
            case '"': o += '"'; break;
            case '\\': o += '\\'; break;
            case '/': o += '/'; break;
            case 'b': o += '\b'; break;
            case 'f': o += '\f'; break;
            case 'n': o += '\n'; break;
            case 'r': o += '\r'; break;
            case 't': o += '\t'; break;
            case 'u':
            {
                unsigned cp = hex4();
                if (cp >= 0xD800 && cp < 0xDC00)
                {
                    if (pos_ + 2 > t_.size() || t_[pos_] != '\\'
                            || t_[pos_ + 1] != 'u')
                        fail("unpaired surrogate");
                    pos_ += 2;
                    unsigned lo = hex4();
                    if (lo < 0xDC00 || lo >= 0xE000)
                        fail("invalid surrogate pair");
                    cp = 0x10000 + ((cp - 0xD800) << 10) + (lo - 0xDC00);
                }
                else if (cp >= 0xDC00 && cp < 0xE000)
                    fail("unpaired surrogate");
                utf8(o, cp);
                break;
            }
            default:
                fail("invalid escape");
            }
        }
    }

    static bool digit(char c) { return c >= '0' && c <= '9'; }

    JsonValue number()
    {
        const size_t start = pos_;
        bool neg = false, frac = false;
        if (peek() == '-') { neg = true; ++pos_; }
        if (at_end() || !digit(peek()))
            fail("invalid number");
        if (peek() == '0')
            ++pos_;
        else
            while (!at_end() && digit(peek())) ++pos_;
        if (!at_end() && peek() == '.')
        {
            frac = true;
            ++pos_;
            if (at_end() || !digit(peek()))
                fail("invalid number: digit expected after '.'");
            while (!at_end() && digit(peek())) ++pos_;
        }
        if (!at_end() && (peek() == 'e' || peek() == 'E'))
        {
            frac = true;
            ++pos_;
            if (!at_end() && (peek() == '+' || peek() == '-')) ++pos_;
            if (at_end() || !digit(peek()))
                fail("invalid number: digit expected in exponent");
            while (!at_end() && digit(peek())) ++pos_;
        }
        const std::string tok = t_.substr(start, pos_ - start);
        JsonValue v;
        if (!frac)
        {
            errno = 0;
            if (neg)
            {
                long long x = std::strtoll(tok.c_str(), nullptr, 10);
                if (errno == 0) { v.type_ = JsonValue::Type::Int; v.i_ = x; return v; }
            }
            else
            {
                unsigned long long x = std::strtoull(tok.c_str(), nullptr, 10);
                if (errno == 0) { v.type_ = JsonValue::Type::UInt; v.u_ = x; return v; }
            }
        }
        v.type_ = JsonValue::Type::Float;
        v.d_ = std::strtod(tok.c_str(), nullptr);
        if (!std::isfinite(v.d_))
            fail("number out of range");
        return v;
    }

    JsonValue value(int depth)
    {
        if (depth > 256)
            fail("nesting too deep");
        ws();
        if (at_end())
            fail("unexpected end of input");
        JsonValue v;
        const char c = peek();
        if (c == '{')
        {
            ++pos_;
            v.type_ = JsonValue::Type::Object;
            v.obj_ = std::make_shared<std::map<std::string, JsonValue>>();
            ws();
            if (!at_end() && peek() == '}') { ++pos_; return v; }
            for (;;)
            {
                ws();
                std::string k = string_lit();
                ws();
                expect(':');
                (*v.obj_)[k] = value(depth + 1);
                ws();
                if (!at_end() && peek() == ',') { ++pos_; continue; }
                expect('}');
                return v;
            }
        }
        if (c == '[')
        {
            ++pos_;
            v.type_ = JsonValue::Type::Array;
            v.arr_ = std::make_shared<std::vector<JsonValue>>();
            ws();
            if (!at_end() && peek() == ']') { ++pos_; return v; }
            for (;;)
            {
                v.arr_->push_back(value(depth + 1));
                ws();
                if (!at_end() && peek() == ',') { ++pos_; continue; }
                expect(']');
                return v;
            }
        }
        if (c == '"')
        {
            v.type_ = JsonValue::Type::String;
            v.s_ = string_lit();
            return v;
        }
        if (c == '-' || digit(c))
            return number();
        if (t_.compare(pos_, 4, "true") == 0)
        {
            pos_ += 4; v.type_ = JsonValue::Type::Bool; v.b_ = true; return v;
        }
        if (t_.compare(pos_, 5, "false") == 0)
        {
            pos_ += 5; v.type_ = JsonValue::Type::Bool; v.b_ = false; return v;
        }
        if (t_.compare(pos_, 4, "null") == 0)
        {
            pos_ += 4; return v;
        }
        fail(std::string("unexpected character '") + c + "'");
    }
};

JsonValue JsonValue::parse(const std::string& text)
{
    return JsonReader(text).document();
}

int64_t JsonValue::intValue(const std::string& what) const
{
    if (type_ == Type::Int) return i_;
    if (type_ == Type::UInt) return (int64_t)u_;
    throw FlameError(what + ": type is not int");
}

double JsonValue::floatValue(const std::string& what) const
{
    if (type_ == Type::Int) return (double)i_;
    if (type_ == Type::UInt) return (double)u_;
    if (type_ == Type::Float) return d_;
    throw FlameError(what + ": type is not float");
}

const std::string& JsonValue::stringValue(const std::string& what) const
{
    if (type_ != Type::String)
        throw FlameError(what + ": type is not string");
    return s_;
}

const std::vector<JsonValue>& JsonValue::arrayValue(const std::string& what) const
{
    if (type_ != Type::Array)
        throw FlameError(what + ": type is not array");
    return *arr_;
}

bool JsonValue::has(const std::string& key) const
{
    return type_ == Type::Object && obj_->count(key) != 0;
}

const JsonValue& JsonValue::at(const std::string& key, const std::string& what) const
{
    if (type_ != Type::Object)
        throw FlameError(what + ": not an object");
    auto it = obj_->find(key);
    if (it == obj_->end())
        throw FlameError(what + ": key does not exist: " + key);
    return it->second;
}

static void dump_str(std::ostringstream& os, const std::string& s)
{
    os << '"';
    for (unsigned char c : s)
    {
        if (c == '"') os << "\\\"";
        else if (c == '\\') os << "\\\\";
        else if (c == '\n') os << "\\n";
        else if (c == '\t') os << "\\t";
        else if (c == '\r') os << "\\r";
        else if (c < 0x20)
        {
            char b[8];
            std::snprintf(b, sizeof b, "\\u%04x", c);
            os << b;
        }
        else os << (char)c;
    }
    os << '"';
}

void JsonValue::dumpTo(std::ostringstream& os) const
{
    switch (type_)
    {
    case Type::Null: os << "null"; return;
    case Type::Bool: os << (b_ ? "true" : "false"); return;
    case Type::Int: os << i_; return;
    case Type::UInt: os << u_; return;
    case Type::Float:
    {
        char b[32];
        std::snprintf(b, sizeof b, "%.17g", d_);
        os << b;
        return;
    }
    case Type::String: dump_str(os, s_); return;
    case Type::Array:
    {
        os << '[';
        for (size_t k = 0; k < arr_->size(); ++k)
        {
            if (k) os << ',';
            (*arr_)[k].dumpTo(os);
        }
        os << ']';
        return;
    }
    case Type::Object:
    {
        os << '{';
        bool first = true;
        for (const auto& kv : *obj_)
        {
            if (!first) os << ',';
            first = false;
            dump_str(os, kv.first);
            os << ':';
            kv.second.dumpTo(os);
        }
        os << '}';
        return;
    }
    }
}

std::string JsonValue::dump() const
{
    std::ostringstream os;
    dumpTo(os);
    return os.str();
}

} // namespace ffr
