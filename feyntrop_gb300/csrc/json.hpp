// Minimal JSON value, parser and writer for feyntrop's low-level interface
// (the 8-key input object of srcs/feyntrop.cpp:25-26 and the result object of
// srcs/feyntrop.cpp:271-278).  Numbers are kept as double plus, when the text is
// an integer, the exact 64-bit value (N and seed need all 64 bits).
#pragma once

#include <cstdint>
#include <map>
#include <memory>
#include <stdexcept>
#include <string>
#include <vector>

namespace ftj {

struct value {
    enum kind_t { null_k, bool_k, number_k, string_k, array_k, object_k } kind = null_k;
    bool b = false;
    double num = 0;
    bool is_integer = false;
    bool negative = false;
    uint64_t uint_value = 0;   // magnitude when is_integer
    std::string str;
    std::vector<value> arr;
    std::map<std::string, value> obj;

    bool is_number() const { return kind == number_k; }
    bool is_array() const { return kind == array_k; }
    bool is_object() const { return kind == object_k; }
    size_t size() const { return kind == array_k ? arr.size() : (kind == object_k ? obj.size() : 0); }
    bool contains(const std::string& k) const { return kind == object_k && obj.count(k); }
    const value& operator[](size_t i) const { return arr.at(i); }
    const value& operator[](const std::string& k) const { return obj.at(k); }
};

value parse(const std::string& text);   // throws std::invalid_argument on malformed text

// conversions with the semantics of a JSON number assigned to the C++ type
uint64_t as_u64(const value& v);
int as_int(const value& v);

std::string number(double x);            // shortest round-trip decimal, "NaN" as null
}  // namespace ftj
