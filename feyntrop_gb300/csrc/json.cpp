#include "json.hpp"

#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>

namespace ftj {
namespace {

struct parser {
    const std::string& s;
    size_t i = 0;

    [[noreturn]] void fail(const char* what)
    {
        throw std::invalid_argument(std::string("json parse error: ") + what + " at offset " + std::to_string(i));
    }
    void ws()
    {
        while (i < s.size() && (s[i] == ' ' || s[i] == '\t' || s[i] == '\n' || s[i] == '\r')) i++;
    }
    bool lit(const char* w)
    {
        size_t n = std::strlen(w);
        if (s.compare(i, n, w) == 0) {
            i += n;
            return true;
        }
        return false;
    }
    value parse_value(int depth)
    {
        if (depth > 64) fail("nesting too deep");
        ws();
        if (i >= s.size()) fail("unexpected end");
        value v;
        char c = s[i];
        if (c == '{') {
            v.kind = value::object_k;
            i++;
            ws();
            if (i < s.size() && s[i] == '}') {
                i++;
                return v;
            }
            while (true) {
                ws();
                if (i >= s.size() || s[i] != '"') fail("expected key");
                std::string k = parse_string();
                ws();
                if (i >= s.size() || s[i] != ':') fail("expected ':'");
                i++;
                v.obj[k] = parse_value(depth + 1);
                ws();
                if (i < s.size() && s[i] == ',') {
                    i++;
                    continue;
                }
                if (i < s.size() && s[i] == '}') {
                    i++;
                    return v;
                }
                fail("expected ',' or '}'");
            }
        }
        if (c == '[') {
            v.kind = value::array_k;
            i++;
            ws();
            if (i < s.size() && s[i] == ']') {
                i++;
                return v;
            }
            while (true) {
                v.arr.push_back(parse_value(depth + 1));
                ws();
                if (i < s.size() && s[i] == ',') {
                    i++;
                    continue;
                }
                if (i < s.size() && s[i] == ']') {
                    i++;
                    return v;
                }
                fail("expected ',' or ']'");
            }
        }
        if (c == '"') {
            v.kind = value::string_k;
            v.str = parse_string();
            return v;
        }
        if (lit("true")) {
            v.kind = value::bool_k;
            v.b = true;
            return v;
        }
        if (lit("false")) {
            v.kind = value::bool_k;
            return v;
        }
        if (lit("null")) return v;
        return parse_number();
    }
    std::string parse_string()
    {
        std::string out;
        i++;  // opening quote
        while (i < s.size() && s[i] != '"') {
            char c = s[i++];
            if (c == '\\') {
                if (i >= s.size()) fail("bad escape");
                char e = s[i++];
                switch (e) {
                case 'n': out += '\n'; break;
                case 't': out += '\t'; break;
                case 'r': out += '\r'; break;
                case 'b': out += '\b'; break;
                case 'f': out += '\f'; break;
                case 'u':
                    if (i + 4 > s.size()) fail("bad unicode escape");
                    out += '?';
                    i += 4;
                    break;
                default: out += e;
                }
            } else {
                out += c;
            }
        }
        if (i >= s.size()) fail("unterminated string");
        i++;
        return out;
    }
    value parse_number()
    {
        size_t start = i;
        if (i < s.size() && (s[i] == '-' || s[i] == '+')) i++;
        bool integer = true;
        while (i < s.size()) {
            char c = s[i];
            if (c >= '0' && c <= '9') {
                i++;
            } else if (c == '.' || c == 'e' || c == 'E' || c == '+' || c == '-') {
                integer = false;
                i++;
            } else {
                break;
            }
        }
        if (i == start) fail("unexpected character");
        std::string t = s.substr(start, i - start);
        if (t == "NaN" || t == "-") fail("bad number");
        value v;
        v.kind = value::number_k;
        char* end = nullptr;
        v.num = std::strtod(t.c_str(), &end);
        if (!end || *end) fail("bad number");
        if (integer) {
            const char* digits = t.c_str();
            v.negative = digits[0] == '-';
            if (digits[0] == '-' || digits[0] == '+') digits++;
            errno = 0;
            unsigned long long u = std::strtoull(digits, &end, 10);
            if (errno == 0 && end && !*end) {
                v.is_integer = true;
                v.uint_value = u;
            }
        }
        return v;
    }
};

}  // namespace

value parse(const std::string& text)
{
    parser p{text};
    value v = p.parse_value(0);
    p.ws();
    if (p.i != text.size()) p.fail("trailing characters");
    return v;
}

uint64_t as_u64(const value& v)
{
    if (v.is_integer && !v.negative) return v.uint_value;
    if (v.is_integer && v.negative) return (uint64_t)(-(int64_t)v.uint_value);
    // a floating JSON number (e.g. 1e7) assigned to an unsigned 64-bit integer
    if (v.num < 0) return (uint64_t)(int64_t)v.num;
    return (uint64_t)v.num;
}

int as_int(const value& v)
{
    if (v.is_integer) return v.negative ? -(int)v.uint_value : (int)v.uint_value;
    return (int)v.num;
}

std::string number(double x)
{
    if (std::isnan(x) || std::isinf(x)) return "null";
    char buf[40];
    for (int prec = 15; prec <= 17; prec++) {
        std::snprintf(buf, sizeof buf, "%.*g", prec, x);
        if (std::strtod(buf, nullptr) == x) break;
    }
    std::string s = buf;
    if (s.find_first_of(".eEn") == std::string::npos) s += ".0";
    return s;
}

}  // namespace ftj
