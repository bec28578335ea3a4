// jsonlite.cpp - implementation of the ordered JSON value, text parser/printer and BJData writer.
#include "jsonlite.h"

#include <algorithm>
#include <cerrno>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <limits>

namespace umcx {
namespace js {

static_assert(sizeof(float) == 4 && sizeof(double) == 8, "IEEE types expected");

Value Value::integer(int64_t v) {
    Value r;
    r.t_ = Type::Int;
    r.i_ = v;
    r.u_ = static_cast<uint64_t>(v);
    return r;
}
Value Value::array() {
    Value r;
    r.t_ = Type::Array;
    return r;
}
Value Value::object() {
    Value r;
    r.t_ = Type::Object;
    return r;
}
Value Value::packed(char marker, const void* data, size_t count) {
    if (marker != 'd' && marker != 'l') throw type_error("packed array: unsupported element type");
    Value r;
    r.t_ = Type::Packed;
    r.pk_ = marker;
    r.raw_.assign(static_cast<const char*>(data), count * 4);
    return r;
}

const char* Value::type_name() const {
    switch (t_) {
        case Type::Null: return "null";
        case Type::Bool: return "boolean";
        case Type::Int:
        case Type::Uint:
        case Type::Float: return "number";
        case Type::String: return "string";
        case Type::Array:
        case Type::Packed: return "array";
        case Type::Object: return "object";
    }
    return "unknown";
}

double Value::as_double() const {
    switch (t_) {
        case Type::Int: return static_cast<double>(i_);
        case Type::Uint: return static_cast<double>(u_);
        case Type::Float: return d_;
        case Type::Bool: return b_ ? 1.0 : 0.0;
        default: throw type_error(std::string("type must be number, but is ") + type_name());
    }
}
int64_t Value::as_int64() const {
    switch (t_) {
        case Type::Int: return i_;
        case Type::Uint: return static_cast<int64_t>(u_);
        case Type::Float: return static_cast<int64_t>(d_);
        case Type::Bool: return b_ ? 1 : 0;
        default: throw type_error(std::string("type must be number, but is ") + type_name());
    }
}
uint64_t Value::as_uint64() const {
    switch (t_) {
        case Type::Int: return static_cast<uint64_t>(i_);
        case Type::Uint: return u_;
        case Type::Float: return static_cast<uint64_t>(d_);
        case Type::Bool: return b_ ? 1 : 0;
        default: throw type_error(std::string("type must be number, but is ") + type_name());
    }
}
const std::string& Value::as_string() const {
    if (t_ != Type::String) throw type_error(std::string("type must be string, but is ") + type_name());
    return s_;
}
bool Value::as_bool() const {
    if (t_ == Type::Bool) return b_;
    throw type_error(std::string("type must be boolean, but is ") + type_name());
}

size_t Value::size() const {
    switch (t_) {
        case Type::Null: return 0;
        case Type::Array: return a_.size();
        case Type::Packed: return raw_.size() / 4;
        case Type::Object: return o_.size();
        default: return 1;
    }
}

const Value* Value::find(const std::string& key) const {
    if (t_ != Type::Object) return nullptr;
    for (const auto& m : o_)
        if (m.first == key) return &m.second;
    return nullptr;
}
Value* Value::find(const std::string& key) {
    if (t_ != Type::Object) return nullptr;
    for (auto& m : o_)
        if (m.first == key) return &m.second;
    return nullptr;
}
Value& Value::operator[](const std::string& key) {
    if (t_ == Type::Null) t_ = Type::Object;
    if (t_ != Type::Object) throw type_error(std::string("cannot use operator[] with a string argument with ") + type_name());
    for (auto& m : o_)
        if (m.first == key) return m.second;
    o_.emplace_back(key, Value());
    return o_.back().second;
}
const Value& Value::at(const std::string& key) const {
    const Value* v = find(key);
    if (!v) throw type_error("key '" + key + "' not found");
    return *v;
}
Value& Value::operator[](size_t i) {
    if (t_ == Type::Null) t_ = Type::Array;
    if (t_ != Type::Array) throw type_error(std::string("cannot use operator[] with a numeric argument with ") + type_name());
    if (i >= a_.size()) a_.resize(i + 1);
    return a_[i];
}
const Value& Value::operator[](size_t i) const { return at(i); }
const Value& Value::at(size_t i) const {
    if (t_ != Type::Array) throw type_error(std::string("cannot use at() with ") + type_name());
    if (i >= a_.size()) throw type_error("array index " + std::to_string(i) + " is out of range");
    return a_[i];
}
void Value::push_back(Value v) {
    if (t_ == Type::Null) t_ = Type::Array;
    if (t_ != Type::Array) throw type_error(std::string("cannot use push_back() with ") + type_name());
    a_.push_back(std::move(v));
}
const std::vector<Value>& Value::items() const {
    if (t_ != Type::Array) throw type_error(std::string("not an array: ") + type_name());
    return a_;
}
const std::vector<Value::Member>& Value::members() const {
    if (t_ != Type::Object) throw type_error(std::string("not an object: ") + type_name());
    return o_;
}
std::vector<Value::Member>& Value::members() {
    if (t_ != Type::Object) throw type_error(std::string("not an object: ") + type_name());
    return o_;
}
const Value::Member& Value::front_member() const {
    if (t_ != Type::Object || o_.empty()) throw type_error("front_member() of an empty or non-object value");
    return o_.front();
}

double Value::value(const std::string& key, double dflt) const {
    const Value* v = find(key);
    return v ? v->as_double() : dflt;
}
int64_t Value::value_int(const std::string& key, int64_t dflt) const {
    const Value* v = find(key);
    return v ? v->as_int64() : dflt;
}
std::string Value::value(const std::string& key, const std::string& dflt) const {
    const Value* v = find(key);
    return v ? v->as_string() : dflt;
}

Value& Value::pointer(const std::string& ptr) {
    if (ptr.empty()) return *this;
    if (ptr[0] != '/') throw parse_error("JSON pointer must start with '/': " + ptr);
    Value* cur = this;
    size_t pos = 1;
    while (true) {
        size_t next = ptr.find('/', pos);
        std::string tok = ptr.substr(pos, next == std::string::npos ? std::string::npos : next - pos);
        std::string key;
        for (size_t k = 0; k < tok.size(); k++) {  // ~1 -> '/', ~0 -> '~'
            if (tok[k] == '~' && k + 1 < tok.size()) {
                key += tok[k + 1] == '1' ? '/' : '~';
                k++;
            } else {
                key += tok[k];
            }
        }
        if (cur->t_ == Type::Array) {
            cur = &(*cur)[static_cast<size_t>(std::strtoull(key.c_str(), nullptr, 10))];
        } else {
            cur = &(*cur)[key];
        }
        if (next == std::string::npos) break;
        pos = next + 1;
    }
    return *cur;
}

void Value::update(const Value& other, bool merge_objects) {
    if (t_ == Type::Null) t_ = Type::Object;
    if (t_ != Type::Object || other.t_ != Type::Object)
        throw type_error(std::string("cannot use update() with ") + type_name());
    for (const auto& m : other.o_) {
        Value* mine = find(m.first);
        if (merge_objects && mine && mine->t_ == Type::Object && m.second.t_ == Type::Object) {
            mine->update(m.second, true);
        } else {
            (*this)[m.first] = m.second;
        }
    }
}

void Value::sort_keys() {
    if (t_ == Type::Object) {
        std::stable_sort(o_.begin(), o_.end(), [](const Member& a, const Member& b) { return a.first < b.first; });
        for (auto& m : o_) m.second.sort_keys();
    } else if (t_ == Type::Array) {
        for (auto& e : a_) e.sort_keys();
    }
}

bool Value::operator==(const Value& o) const {
    if (is_number() && o.is_number()) {
        if (t_ == Type::Float || o.t_ == Type::Float) return as_double() == o.as_double();
        if (t_ == Type::Int && o.t_ == Type::Int) return i_ == o.i_;
        if (t_ == Type::Uint && o.t_ == Type::Uint) return u_ == o.u_;
        const Value& s = t_ == Type::Int ? *this : o;
        const Value& u = t_ == Type::Int ? o : *this;
        return s.i_ >= 0 && static_cast<uint64_t>(s.i_) == u.u_;
    }
    if (t_ != o.t_) return false;
    switch (t_) {
        case Type::Null: return true;
        case Type::Bool: return b_ == o.b_;
        case Type::String: return s_ == o.s_;
        case Type::Array: return a_ == o.a_;
        case Type::Packed: return pk_ == o.pk_ && raw_ == o.raw_;
        case Type::Object: return o_ == o.o_;
        default: return false;
    }
}

// ------------------------------------------------------------------ text parser
namespace {
struct Parser {
    const char* p;
    const char* end;
    size_t depth = 0;

    [[noreturn]] void fail(const std::string& what) const {
        throw parse_error("JSON parse error at offset " + std::to_string(static_cast<size_t>(p - begin)) + ": " + what);
    }
    const char* begin;

    void ws() {
        while (p < end && (*p == ' ' || *p == '\t' || *p == '\n' || *p == '\r')) p++;
    }
    bool lit(const char* s) {
        size_t n = std::strlen(s);
        if (static_cast<size_t>(end - p) >= n && std::memcmp(p, s, n) == 0) {
            p += n;
            return true;
        }
        return false;
    }
    static void utf8(std::string& out, uint32_t cp) {
        if (cp < 0x80) {
            out += static_cast<char>(cp);
        } else if (cp < 0x800) {
            out += static_cast<char>(0xC0 | (cp >> 6));
            out += static_cast<char>(0x80 | (cp & 0x3F));
        } else if (cp < 0x10000) {
            out += static_cast<char>(0xE0 | (cp >> 12));
            out += static_cast<char>(0x80 | ((cp >> 6) & 0x3F));
            out += static_cast<char>(0x80 | (cp & 0x3F));
        } else {
            out += static_cast<char>(0xF0 | (cp >> 18));
            out += static_cast<char>(0x80 | ((cp >> 12) & 0x3F));
            out += static_cast<char>(0x80 | ((cp >> 6) & 0x3F));
            out += static_cast<char>(0x80 | (cp & 0x3F));
        }
    }
    uint32_t hex4() {
        if (end - p < 4) fail("truncated \\u escape");
        uint32_t v = 0;
        for (int k = 0; k < 4; k++) {
            char c = *p++;
            v <<= 4;
            if (c >= '0' && c <= '9') v |= static_cast<uint32_t>(c - '0');
            else if (c >= 'a' && c <= 'f') v |= static_cast<uint32_t>(c - 'a' + 10);
            else if (c >= 'A' && c <= 'F') v |= static_cast<uint32_t>(c - 'A' + 10);
            else fail("invalid \\u escape");
        }
        return v;
    }
    std::string str() {
        if (p >= end || *p != '"') fail("expected string");
        p++;
        std::string out;
        while (true) {
            if (p >= end) fail("unterminated string");
            char c = *p++;
            if (c == '"') break;
            if (static_cast<unsigned char>(c) < 0x20) fail("control character in string");
            if (c != '\\') {
                out += c;
                continue;
            }
            if (p >= end) fail("unterminated escape");
            char e = *p++;
            switch (e) {
                case '"': out += '"'; break;
                case '\\': out += '\\'; break;
                case '/': out += '/'; break;
                case 'b': out += '\b'; break;
                case 'f': out += '\f'; break;
                case 'n': out += '\n'; break;
                case 'r': out += '\r'; break;
                case 't': out += '\t'; break;
                case 'u': {
                    uint32_t cp = hex4();
                    if (cp >= 0xD800 && cp <= 0xDBFF) {
                        if (!lit("\\u")) fail("unpaired surrogate");
                        uint32_t lo = hex4();
                        if (lo < 0xDC00 || lo > 0xDFFF) fail("invalid surrogate pair");
                        cp = 0x10000 + ((cp - 0xD800) << 10) + (lo - 0xDC00);
                    }
                    utf8(out, cp);
                    break;
                }
                default: fail("invalid escape");
            }
        }
        return out;
    }
    Value number() {
        const char* s = p;
        bool neg = false, isfloat = false;
        if (p < end && *p == '-') {
            neg = true;
            p++;
        }
        if (p >= end || !(*p >= '0' && *p <= '9')) fail("invalid number");
        if (*p == '0') {
            p++;
        } else {
            while (p < end && *p >= '0' && *p <= '9') p++;
        }
        if (p < end && *p == '.') {
            isfloat = true;
            p++;
            if (p >= end || !(*p >= '0' && *p <= '9')) fail("invalid number");
            while (p < end && *p >= '0' && *p <= '9') p++;
        }
        if (p < end && (*p == 'e' || *p == 'E')) {
            isfloat = true;
            p++;
            if (p < end && (*p == '+' || *p == '-')) p++;
            if (p >= end || !(*p >= '0' && *p <= '9')) fail("invalid number");
            while (p < end && *p >= '0' && *p <= '9') p++;
        }
        std::string tok(s, static_cast<size_t>(p - s));
        if (!isfloat) {
            errno = 0;
            if (neg) {
                long long v = std::strtoll(tok.c_str(), nullptr, 10);
                if (errno == 0) return Value::integer(v);
            } else {
                unsigned long long v = std::strtoull(tok.c_str(), nullptr, 10);
                if (errno == 0) return Value(v);
            }
        }
        return Value(std::strtod(tok.c_str(), nullptr));
    }
    Value value() {
        if (++depth > 512) fail("nesting too deep");
        ws();
        if (p >= end) fail("unexpected end of input");
        Value r;
        char c = *p;
        if (c == '{') {
            p++;
            r = Value::object();
            ws();
            if (p < end && *p == '}') {
                p++;
            } else {
                while (true) {
                    ws();
                    std::string k = str();
                    ws();
                    if (p >= end || *p != ':') fail("expected ':'");
                    p++;
                    Value v = value();
                    Value* existing = r.find(k);
                    if (existing) *existing = std::move(v);
                    else r.members().emplace_back(std::move(k), std::move(v));
                    ws();
                    if (p < end && *p == ',') {
                        p++;
                        continue;
                    }
                    if (p < end && *p == '}') {
                        p++;
                        break;
                    }
                    fail("expected ',' or '}'");
                }
            }
        } else if (c == '[') {
            p++;
            r = Value::array();
            ws();
            if (p < end && *p == ']') {
                p++;
            } else {
                while (true) {
                    r.push_back(value());
                    ws();
                    if (p < end && *p == ',') {
                        p++;
                        continue;
                    }
                    if (p < end && *p == ']') {
                        p++;
                        break;
                    }
                    fail("expected ',' or ']'");
                }
            }
        } else if (c == '"') {
            r = Value(str());
        } else if (lit("true")) {
            r = Value(true);
        } else if (lit("false")) {
            r = Value(false);
        } else if (lit("null")) {
            r = Value();
        } else {
            r = number();
        }
        depth--;
        return r;
    }
};
}  // namespace

Value Value::parse(const std::string& text) {
    Parser ps;
    ps.begin = text.data();
    ps.p = text.data();
    ps.end = text.data() + text.size();
    Value v = ps.value();
    ps.ws();
    if (ps.p != ps.end) ps.fail("unexpected trailing characters");
    return v;
}

// ------------------------------------------------------------------ text printer
std::string format_double(double v) {
    if (std::isnan(v) || std::isinf(v)) return "null";
    if (v == 0.0) return std::signbit(v) ? "-0.0" : "0.0";
    char buf[40];
    int prec = 1;
    for (; prec <= 17; prec++) {
        std::snprintf(buf, sizeof(buf), "%.*e", prec - 1, v);
        if (std::strtod(buf, nullptr) == v) break;
    }
    // split "d.ddde[+-]XX" into digits and decimal exponent
    std::string s(buf);
    bool neg = s[0] == '-';
    if (neg) s.erase(0, 1);
    size_t epos = s.find('e');
    int e10 = std::atoi(s.c_str() + epos + 1);
    std::string digits;
    for (size_t k = 0; k < epos; k++)
        if (s[k] != '.') digits += s[k];
    while (digits.size() > 1 && digits.back() == '0') digits.pop_back();
    const int k = static_cast<int>(digits.size());
    const int n = e10 + 1;  // position of the decimal point relative to the digits
    std::string out = neg ? "-" : "";
    const int min_exp = -4, max_exp = 15;
    if (k <= n && n <= max_exp) {
        out += digits + std::string(static_cast<size_t>(n - k), '0') + ".0";
    } else if (0 < n && n <= max_exp) {
        out += digits.substr(0, static_cast<size_t>(n)) + "." + digits.substr(static_cast<size_t>(n));
    } else if (min_exp < n && n <= 0) {
        out += "0." + std::string(static_cast<size_t>(-n), '0') + digits;
    } else {
        out += digits.substr(0, 1);
        if (k > 1) out += "." + digits.substr(1);
        int ex = n - 1;
        char eb[16];
        std::snprintf(eb, sizeof(eb), "e%c%02d", ex < 0 ? '-' : '+', ex < 0 ? -ex : ex);
        out += eb;
    }
    return out;
}

static void dump_string(std::string& out, const std::string& s) {
    out += '"';
    for (unsigned char c : s) {
        switch (c) {
            case '"': out += "\\\""; break;
            case '\\': out += "\\\\"; break;
            case '\b': out += "\\b"; break;
            case '\f': out += "\\f"; break;
            case '\n': out += "\\n"; break;
            case '\r': out += "\\r"; break;
            case '\t': out += "\\t"; break;
            default:
                if (c < 0x20) {
                    char b[8];
                    std::snprintf(b, sizeof(b), "\\u%04x", c);
                    out += b;
                } else {
                    out += static_cast<char>(c);
                }
        }
    }
    out += '"';
}

void Value::dump_to(std::string& out, int indent, int level) const {
    const bool pretty = indent >= 0;
    const std::string nl = pretty ? "\n" : "";
    auto pad = [&](int lv) { return pretty ? std::string(static_cast<size_t>(indent * lv), ' ') : std::string(); };
    switch (t_) {
        case Type::Null: out += "null"; break;
        case Type::Bool: out += b_ ? "true" : "false"; break;
        case Type::Int: out += std::to_string(i_); break;
        case Type::Uint: out += std::to_string(u_); break;
        case Type::Float: out += format_double(d_); break;
        case Type::String: dump_string(out, s_); break;
        case Type::Packed:
        case Type::Array: {
            size_t n = size();
            if (n == 0) {
                out += "[]";
                break;
            }
            out += "[" + nl;
            for (size_t k = 0; k < n; k++) {
                out += pad(level + 1);
                if (t_ == Type::Packed) {
                    if (pk_ == 'd') {
                        float f;
                        std::memcpy(&f, raw_.data() + 4 * k, 4);
                        out += format_double(static_cast<double>(f));
                    } else {
                        int32_t iv;
                        std::memcpy(&iv, raw_.data() + 4 * k, 4);
                        out += std::to_string(iv);
                    }
                } else {
                    a_[k].dump_to(out, indent, level + 1);
                }
                if (k + 1 < n) out += pretty ? ",\n" : ",";
            }
            out += nl + pad(level) + "]";
            break;
        }
        case Type::Object: {
            if (o_.empty()) {
                out += "{}";
                break;
            }
            out += "{" + nl;
            for (size_t k = 0; k < o_.size(); k++) {
                out += pad(level + 1);
                dump_string(out, o_[k].first);
                out += pretty ? ": " : ":";
                o_[k].second.dump_to(out, indent, level + 1);
                if (k + 1 < o_.size()) out += pretty ? ",\n" : ",";
            }
            out += nl + pad(level) + "}";
            break;
        }
    }
}

std::string Value::dump(int indent) const {
    std::string out;
    dump_to(out, indent, 0);
    return out;
}

// ------------------------------------------------------------------ BJData writer
// Integer markers of BJData Draft 2, smallest type that holds the value, in the order
// int8 'i', uint8 'U', int16 'I', uint16 'u', int32 'l', uint32 'm', int64 'L', uint64 'M'.
static char bj_int_marker_signed(int64_t v) {
    if (v >= -128 && v <= 127) return 'i';
    if (v >= 0 && v <= 255) return 'U';
    if (v >= -32768 && v <= 32767) return 'I';
    if (v >= 0 && v <= 65535) return 'u';
    if (v >= INT32_MIN && v <= INT32_MAX) return 'l';
    if (v >= 0 && v <= static_cast<int64_t>(UINT32_MAX)) return 'm';
    return 'L';
}
static char bj_int_marker_unsigned(uint64_t v) {
    if (v <= 127u) return 'i';
    if (v <= 255u) return 'U';
    if (v <= 32767u) return 'I';
    if (v <= 65535u) return 'u';
    if (v <= static_cast<uint64_t>(INT32_MAX)) return 'l';
    if (v <= UINT32_MAX) return 'm';
    if (v <= static_cast<uint64_t>(INT64_MAX)) return 'L';
    return 'M';
}
template <class T>
static void bj_raw(std::string& out, T v) {
    char b[sizeof(T)];
    std::memcpy(b, &v, sizeof(T));  // little-endian hosts only (x86-64, aarch64)
    out.append(b, sizeof(T));
}
static void bj_int_payload(std::string& out, char m, uint64_t bits) {
    switch (m) {
        case 'i': bj_raw(out, static_cast<int8_t>(bits)); break;
        case 'U': bj_raw(out, static_cast<uint8_t>(bits)); break;
        case 'I': bj_raw(out, static_cast<int16_t>(bits)); break;
        case 'u': bj_raw(out, static_cast<uint16_t>(bits)); break;
        case 'l': bj_raw(out, static_cast<int32_t>(bits)); break;
        case 'm': bj_raw(out, static_cast<uint32_t>(bits)); break;
        case 'L': bj_raw(out, static_cast<int64_t>(bits)); break;
        default: bj_raw(out, static_cast<uint64_t>(bits)); break;
    }
}
static void bj_count(std::string& out, uint64_t n) {
    char m = bj_int_marker_unsigned(n);
    out += m;
    bj_int_payload(out, m, n);
}

char Value::bj_marker() const {
    switch (t_) {
        case Type::Null: return 'Z';
        case Type::Bool: return b_ ? 'T' : 'F';
        case Type::Int: return bj_int_marker_signed(i_);
        case Type::Uint: return bj_int_marker_unsigned(u_);
        case Type::Float: return 'D';
        case Type::String: return 'S';
        case Type::Array:
        case Type::Packed: return '[';
        case Type::Object: return '{';
    }
    return 'Z';
}

// JData annotated array {_ArrayType_, _ArraySize_, _ArrayData_} -> BJData ND-array; returns false when the object
// does not qualify (then it is written as a plain object)
bool Value::bj_ndarray(std::string& out) const {
    if (t_ != Type::Object || o_.size() != 3) return false;
    const Value* ty = find("_ArrayType_");
    const Value* sz = find("_ArraySize_");
    const Value* da = find("_ArrayData_");
    if (!ty || !sz || !da || !ty->is_string() || !sz->is_array() || !da->is_array()) return false;
    static const struct { const char* name; char m; } types[] = {
        {"uint8", 'U'}, {"int8", 'i'}, {"uint16", 'u'}, {"int16", 'I'},  {"uint32", 'm'}, {"int32", 'l'},
        {"uint64", 'M'}, {"int64", 'L'}, {"single", 'd'}, {"double", 'D'}, {"char", 'C'}};
    char m = 0;
    for (const auto& t : types)
        if (ty->s_ == t.name) m = t.m;
    if (!m) return false;
    uint64_t len = 1;
    for (size_t k = 0; k < sz->size(); k++) len *= sz->at(k).as_uint64();
    if (len != da->size()) return false;
    out += '[';
    out += '$';
    out += m;
    out += '#';
    sz->bj_write(out, true);
    if (da->t_ == Type::Packed) {
        if (da->pk_ != m) throw type_error("packed array type does not match _ArrayType_");
        out += da->raw_;
        return true;
    }
    for (const Value& e : da->a_) {
        switch (m) {
            case 'U': bj_raw(out, static_cast<uint8_t>(e.as_uint64())); break;
            case 'i': bj_raw(out, static_cast<int8_t>(e.as_int64())); break;
            case 'u': bj_raw(out, static_cast<uint16_t>(e.as_uint64())); break;
            case 'I': bj_raw(out, static_cast<int16_t>(e.as_int64())); break;
            case 'm': bj_raw(out, static_cast<uint32_t>(e.as_uint64())); break;
            case 'l': bj_raw(out, static_cast<int32_t>(e.as_int64())); break;
            case 'M': bj_raw(out, static_cast<uint64_t>(e.as_uint64())); break;
            case 'L': bj_raw(out, static_cast<int64_t>(e.as_int64())); break;
            case 'd': bj_raw(out, static_cast<float>(e.as_double())); break;
            case 'D': bj_raw(out, static_cast<double>(e.as_double())); break;
            default: bj_raw(out, static_cast<uint8_t>(e.as_uint64())); break;
        }
    }
    return true;
}

void Value::bj_write(std::string& out, bool with_marker) const {
    switch (t_) {
        case Type::Null:
        case Type::Bool:
            if (with_marker) out += bj_marker();
            break;
        case Type::Int: {
            char m = bj_marker();
            if (with_marker) out += m;
            bj_int_payload(out, m, static_cast<uint64_t>(i_));
            break;
        }
        case Type::Uint: {
            char m = bj_marker();
            if (with_marker) out += m;
            bj_int_payload(out, m, u_);
            break;
        }
        case Type::Float:
            if (with_marker) out += 'D';
            bj_raw(out, d_);
            break;
        case Type::String:
            if (with_marker) out += 'S';
            bj_count(out, s_.size());
            out += s_;
            break;
        case Type::Packed: {
            if (with_marker) out += '[';
            out += '$';
            out += pk_;
            out += '#';
            bj_count(out, size());
            out += raw_;
            break;
        }
        case Type::Array: {
            if (with_marker) out += '[';
            bool typed = false;
            char first = 0;
            if (!a_.empty()) {
                first = a_.front().bj_marker();
                typed = true;
                for (size_t k = 1; k < a_.size() && typed; k++) typed = a_[k].bj_marker() == first;
                // BJData forbids these markers as an optimised element type
                if (std::strchr("[{SHTFNZ", first)) typed = false;
            }
            if (typed) {
                out += '$';
                out += first;
            }
            out += '#';
            bj_count(out, a_.size());
            for (const Value& e : a_) e.bj_write(out, !typed);
            break;
        }
        case Type::Object: {
            if (bj_ndarray(out)) break;
            if (with_marker) out += '{';
            bool typed = false;
            char first = 0;
            if (!o_.empty()) {
                first = o_.front().second.bj_marker();
                typed = true;
                for (size_t k = 1; k < o_.size() && typed; k++) typed = o_[k].second.bj_marker() == first;
                if (std::strchr("[{SHTFNZ", first)) typed = false;
            }
            if (typed) {
                out += '$';
                out += first;
            }
            out += '#';
            bj_count(out, o_.size());
            for (const Member& m : o_) {
                bj_count(out, m.first.size());
                out += m.first;
                m.second.bj_write(out, !typed);
            }
            break;
        }
    }
}

void Value::to_bjdata(std::string& out) const { bj_write(out, true); }

}  // namespace js
}  // namespace umcx
