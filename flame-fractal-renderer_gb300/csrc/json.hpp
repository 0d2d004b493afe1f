// Read-only JSON document model for flame files.
//
// Accept/reject behaviour follows the reference's JSON front end, which
// parses with comments allowed (src/utils/json.cpp:15-23) and exposes typed
// accessors that throw on a type mismatch (src/utils/json.cpp:87-147):
//   * // and /* */ comments count as whitespace;
//   * integers (no '.', 'e', 'E') stay integers, everything else is a double
//     converted with strtod (correctly rounded);
//   * a duplicate key keeps the last value; trailing garbage is an error.
#pragma once

#include <cstdint>
#include <map>
#include <sstream>
#include <memory>
#include <stdexcept>
#include <string>
#include <vector>

namespace ffr {

// Parse or validation error (the reference's JsonError, json.hpp:12-24).
class FlameError : public std::runtime_error
{
public:
    explicit FlameError(const std::string& m) : std::runtime_error(m) {}
};

class JsonValue
{
public:
    enum class Type { Null, Bool, Int, UInt, Float, String, Array, Object };

    JsonValue() = default;

    static JsonValue parse(const std::string& text);

    Type type() const { return type_; }
    bool isNull() const { return type_ == Type::Null; }
    bool isBool() const { return type_ == Type::Bool; }
    // the reference's isInt() (is_number_integer: signed or unsigned)
    bool isInt() const { return type_ == Type::Int || type_ == Type::UInt; }
    // the reference's isFloat() (is_number: any number)
    bool isNumber() const { return isInt() || type_ == Type::Float; }
    bool isString() const { return type_ == Type::String; }
    bool isArray() const { return type_ == Type::Array; }
    bool isObject() const { return type_ == Type::Object; }

    // typed accessors; throw FlameError with `what` on a type mismatch
    int64_t intValue(const std::string& what) const;
    double floatValue(const std::string& what) const;
    const std::string& stringValue(const std::string& what) const;
    const std::vector<JsonValue>& arrayValue(const std::string& what) const;

    bool has(const std::string& key) const;
    // object member; throws FlameError("... key does not exist: k")
    const JsonValue& at(const std::string& key, const std::string& what) const;
    // compact text form (for the CLI's "flame:" echo)
    std::string dump() const;

private:
    void dumpTo(std::ostringstream& os) const;

    Type type_ = Type::Null;
    bool b_ = false;
    int64_t i_ = 0;
    uint64_t u_ = 0;
    double d_ = 0.0;
    std::string s_;
    std::shared_ptr<std::vector<JsonValue>> arr_;
    std::shared_ptr<std::map<std::string, JsonValue>> obj_;

    friend class JsonReader;
};

} // namespace ffr
