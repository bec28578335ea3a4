// jsonlite.h - small ordered JSON value with a text parser/printer and a BJData (Draft 2) writer.
//
// The reference front end uses nlohmann::ordered_json (src/umcx.cpp:56) for its input and for its binary
// outputs (json::to_bjdata(..., use_size=true, use_type=true), L703).  This is an independent implementation of
// the subset the front end needs: insertion-ordered objects, number kinds (signed / unsigned / float) kept apart
// the way the input spelled them, numeric conversions that accept booleans, JSON-pointer assignment, recursive
// merge, and a BJData writer whose container optimisation and JData ND-array packing produce the byte layout
// that the reference's .bnii / _detp.jdb files have.
#pragma once

#include <cstdint>
#include <stdexcept>
#include <string>
#include <utility>
#include <vector>

namespace umcx {
namespace js {

struct type_error : std::runtime_error {
    using std::runtime_error::runtime_error;
};
struct parse_error : std::runtime_error {
    using std::runtime_error::runtime_error;
};

enum class Type : uint8_t { Null, Bool, Int, Uint, Float, String, Array, Object, Packed };

class Value {
public:
    using Member = std::pair<std::string, Value>;

    Value() = default;
    Value(std::nullptr_t) {}
    Value(bool v) : t_(Type::Bool), b_(v) {}
    Value(int v) : t_(Type::Int), i_(v), u_(static_cast<uint64_t>(v)) {}
    Value(long v) : t_(Type::Int), i_(v), u_(static_cast<uint64_t>(v)) {}
    Value(long long v) : t_(Type::Int), i_(v), u_(static_cast<uint64_t>(v)) {}
    Value(unsigned v) : t_(Type::Uint), i_(static_cast<int64_t>(v)), u_(v) {}
    Value(unsigned long v) : t_(Type::Uint), i_(static_cast<int64_t>(v)), u_(v) {}
    Value(unsigned long long v) : t_(Type::Uint), i_(static_cast<int64_t>(v)), u_(v) {}
    Value(double v) : t_(Type::Float), d_(v) {}
    Value(float v) : t_(Type::Float), d_(v) {}
    Value(const char* s) : t_(Type::String), s_(s) {}
    Value(std::string s) : t_(Type::String), s_(std::move(s)) {}

    // signed integer that keeps the "signed" kind even when non-negative (nlohmann number_integer)
    static Value integer(int64_t v);
    static Value array();
    static Value object();
    // a numeric array kept packed (large volumes): marker 'd' = float32, 'l' = int32; elements are copied
    static Value packed(char marker, const void* data, size_t count);

    Type type() const { return t_; }
    bool is_null() const { return t_ == Type::Null; }
    bool is_bool() const { return t_ == Type::Bool; }
    bool is_number() const { return t_ == Type::Int || t_ == Type::Uint || t_ == Type::Float; }
    bool is_integer() const { return t_ == Type::Int || t_ == Type::Uint; }
    bool is_string() const { return t_ == Type::String; }
    bool is_array() const { return t_ == Type::Array || t_ == Type::Packed; }
    bool is_object() const { return t_ == Type::Object; }
    const char* type_name() const;

    // numeric conversions (accept numbers and booleans, like nlohmann's arithmetic from_json)
    double as_double() const;
    float as_float() const { return static_cast<float>(as_double()); }
    int64_t as_int64() const;
    uint64_t as_uint64() const;
    int as_int() const { return static_cast<int>(as_int64()); }
    const std::string& as_string() const;
    bool as_bool() const;

    // containers
    size_t size() const;
    bool empty() const { return size() == 0; }
    bool contains(const std::string& key) const { return find(key) != nullptr; }
    const Value* find(const std::string& key) const;
    Value* find(const std::string& key);
    // object access: inserts null when missing (a null value becomes an object first)
    Value& operator[](const std::string& key);
    Value& operator[](const char* key) { return (*this)[std::string(key)]; }
    // const object access: throws when missing
    const Value& at(const std::string& key) const;
    // array access
    Value& operator[](size_t i);
    const Value& operator[](size_t i) const;
    const Value& at(size_t i) const;
    void push_back(Value v);
    const std::vector<Value>& items() const;
    const std::vector<Member>& members() const;
    std::vector<Member>& members();
    // first member of an object (key, value)
    const Member& front_member() const;

    // value(key, default) of nlohmann: member if present, else the default
    double value(const std::string& key, double dflt) const;
    int64_t value_int(const std::string& key, int64_t dflt) const;
    std::string value(const std::string& key, const std::string& dflt) const;

    // JSON pointer ("/a/b/0") write access, creating objects along the way
    Value& pointer(const std::string& ptr);
    // recursive merge of objects (nlohmann update(j, merge_objects=true))
    void update(const Value& other, bool merge_objects = true);
    // order every object's members by key, recursively (the key order of a std::map-backed JSON value)
    void sort_keys();

    static Value parse(const std::string& text);
    std::string dump(int indent = -1) const;
    // BJData Draft 2 with count + type optimisation and JData ND-array packing
    void to_bjdata(std::string& out) const;

    bool operator==(const Value& o) const;
    bool operator!=(const Value& o) const { return !(*this == o); }

private:
    Type t_ = Type::Null;
    bool b_ = false;
    int64_t i_ = 0;
    uint64_t u_ = 0;
    double d_ = 0.0;
    std::string s_;
    std::vector<Value> a_;
    std::vector<Member> o_;
    char pk_ = 0;       // element marker of a packed array
    std::string raw_;   // packed element bytes (little-endian)

    void dump_to(std::string& out, int indent, int level) const;
    void bj_write(std::string& out, bool with_marker) const;
    char bj_marker() const;
    bool bj_ndarray(std::string& out) const;
};

// shortest round-trip text of a double, formatted like nlohmann's serializer
std::string format_double(double v);

}  // namespace js
}  // namespace umcx
