// Minimal JSON reader for cam.json (RFC 8259 subset: objects, arrays,
// strings with escapes, numbers, true/false/null).
//
// Numbers follow the reference's reader (nlohmann::json, used by
// src/file_reader.cu:39-107): an integer literal is kept as a 64-bit integer
// and converted to float directly when a float is asked for, any other number
// is parsed as a double and then rounded to float.
#pragma once

#include <cerrno>
#include <cstdint>
#include <cstdlib>
#include <map>
#include <memory>
#include <stdexcept>
#include <string>
#include <vector>

namespace isti::host
{
struct Json
{
    enum Kind { Null, Bool, Int, Real, String, Array, Object } kind = Null;
    bool b = false;
    int64_t i = 0;
    double d = 0.0;
    std::string s;
    std::vector<Json> items;
    std::map<std::string, Json> fields;

    const Json *find(const std::string &key) const
    {
        if (kind != Object)
            return nullptr;
        const auto it = fields.find(key);
        return it == fields.end() ? nullptr : &it->second;
    }
    const Json &at(const std::string &key) const
    {
        const Json *j = find(key);
        if (!j)
            throw std::runtime_error("cam.json: missing key \"" + key + "\"");
        return *j;
    }
    bool is_number() const { return kind == Int || kind == Real; }
    float as_float() const
    {
        if (kind == Int)
            return static_cast<float>(i);
        if (kind == Real)
            return static_cast<float>(d);
        throw std::runtime_error("cam.json: number expected");
    }
    int as_int() const
    {
        if (kind == Int)
            return static_cast<int>(i);
        if (kind == Real)
            return static_cast<int>(d);
        throw std::runtime_error("cam.json: integer expected");
    }
    bool as_bool() const
    {
        if (kind != Bool)
            throw std::runtime_error("cam.json: boolean expected");
        return b;
    }

    static Json parse(const std::string &text)
    {
        size_t pos = 0;
        Json j = parse_value(text, pos, 0);
        skip_ws(text, pos);
        if (pos != text.size())
            throw std::runtime_error("cam.json: trailing characters");
        return j;
    }

private:
    static void skip_ws(const std::string &t, size_t &p)
    {
        while (p < t.size() && (t[p] == ' ' || t[p] == '\t' || t[p] == '\n' || t[p] == '\r'))
            p++;
    }
    [[noreturn]] static void fail(const char *what, size_t p)
    {
        throw std::runtime_error(std::string("cam.json: ") + what + " at offset " + std::to_string(p));
    }
    static void append_utf8(std::string &out, uint32_t cp)
    {
        if (cp < 0x80)
            out += char(cp);
        else if (cp < 0x800)
        {
            out += char(0xc0 | (cp >> 6));
            out += char(0x80 | (cp & 0x3f));
        }
        else if (cp < 0x10000)
        {
            out += char(0xe0 | (cp >> 12));
            out += char(0x80 | ((cp >> 6) & 0x3f));
            out += char(0x80 | (cp & 0x3f));
        }
        else
        {
            out += char(0xf0 | (cp >> 18));
            out += char(0x80 | ((cp >> 12) & 0x3f));
            out += char(0x80 | ((cp >> 6) & 0x3f));
            out += char(0x80 | (cp & 0x3f));
        }
    }
    static uint32_t hex4(const std::string &t, size_t &p)
    {
        if (p + 4 > t.size())
            fail("bad \\u escape", p);
        uint32_t v = 0;
        for (int k = 0; k < 4; k++)
        {
            const char c = t[p++];
            v <<= 4;
            if (c >= '0' && c <= '9') v |= uint32_t(c - '0');
            else if (c >= 'a' && c <= 'f') v |= uint32_t(c - 'a' + 10);
            else if (c >= 'A' && c <= 'F') v |= uint32_t(c - 'A' + 10);
            else fail("bad \\u escape", p);
        }
        return v;
    }
    static std::string parse_string(const std::string &t, size_t &p)
    {
        if (p >= t.size() || t[p] != '"')
            fail("string expected", p);
        p++;
        std::string out;
        while (p < t.size() && t[p] != '"')
        {
            const char c = t[p++];
            if (static_cast<unsigned char>(c) < 0x20)
                fail("control character in string", p);
            if (c != '\\')
            {
                out += c;
                continue;
            }
            if (p >= t.size())
                fail("bad escape", p);
            const char e = t[p++];
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
                uint32_t cp = hex4(t, p);
                if (cp >= 0xd800 && cp < 0xdc00 && p + 6 <= t.size() && t[p] == '\\' && t[p + 1] == 'u')
                {
                    p += 2;
                    const uint32_t lo = hex4(t, p);
                    if (lo < 0xdc00 || lo >= 0xe000)
                        fail("bad surrogate pair", p);
                    cp = 0x10000 + ((cp - 0xd800) << 10) + (lo - 0xdc00);
                }
                append_utf8(out, cp);
                break;
            }
            default: fail("bad escape", p);
            }
        }
        if (p >= t.size())
            fail("unterminated string", p);
        p++;
        return out;
    }
    static Json parse_number(const std::string &t, size_t &p)
    {
        const size_t start = p;
        if (p < t.size() && t[p] == '-')
            p++;
        if (p >= t.size() || t[p] < '0' || t[p] > '9')
            fail("bad number", p);
        if (t[p] == '0')
            p++;
        else
            while (p < t.size() && t[p] >= '0' && t[p] <= '9')
                p++;
        bool integer = true;
        if (p < t.size() && t[p] == '.')
        {
            integer = false;
            p++;
            if (p >= t.size() || t[p] < '0' || t[p] > '9')
                fail("bad number", p);
            while (p < t.size() && t[p] >= '0' && t[p] <= '9')
                p++;
        }
        if (p < t.size() && (t[p] == 'e' || t[p] == 'E'))
        {
            integer = false;
            p++;
            if (p < t.size() && (t[p] == '+' || t[p] == '-'))
                p++;
            if (p >= t.size() || t[p] < '0' || t[p] > '9')
                fail("bad number", p);
            while (p < t.size() && t[p] >= '0' && t[p] <= '9')
                p++;
        }
        const std::string lit = t.substr(start, p - start);
        Json j;
        if (integer)
        {
            errno = 0;
            const long long v = std::strtoll(lit.c_str(), nullptr, 10);
            if (errno == 0)
            {
                j.kind = Int;
                j.i = v;
                return j;
            }
        }
        j.kind = Real;
        j.d = std::strtod(lit.c_str(), nullptr);
        return j;
    }
    static Json parse_value(const std::string &t, size_t &p, int depth)
    {
        if (depth > 64)
            fail("nesting too deep", p);
        skip_ws(t, p);
        if (p >= t.size())
            fail("value expected", p);
        Json j;
        const char c = t[p];
        if (c == '{')
        {
            j.kind = Object;
            p++;
            skip_ws(t, p);
            if (p < t.size() && t[p] == '}')
            {
                p++;
                return j;
            }
            for (;;)
            {
                skip_ws(t, p);
                std::string key = parse_string(t, p);
                skip_ws(t, p);
                if (p >= t.size() || t[p] != ':')
                    fail("':' expected", p);
                p++;
                j.fields[key] = parse_value(t, p, depth + 1);
                skip_ws(t, p);
                if (p < t.size() && t[p] == ',')
                {
                    p++;
                    continue;
                }
                if (p < t.size() && t[p] == '}')
                {
                    p++;
                    return j;
                }
                fail("',' or '}' expected", p);
            }
        }
        if (c == '[')
        {
            j.kind = Array;
            p++;
            skip_ws(t, p);
            if (p < t.size() && t[p] == ']')
            {
                p++;
                return j;
            }
            for (;;)
            {
                j.items.push_back(parse_value(t, p, depth + 1));
                skip_ws(t, p);
                if (p < t.size() && t[p] == ',')
                {
                    p++;
                    continue;
                }
                if (p < t.size() && t[p] == ']')
                {
                    p++;
                    return j;
                }
                fail("',' or ']' expected", p);
            }
        }
        if (c == '"')
        {
            j.kind = String;
            j.s = parse_string(t, p);
            return j;
        }
        if (t.compare(p, 4, "true") == 0)
        {
            p += 4;
            j.kind = Bool;
            j.b = true;
            return j;
        }
        if (t.compare(p, 5, "false") == 0)
        {
            p += 5;
            j.kind = Bool;
            return j;
        }
        if (t.compare(p, 4, "null") == 0)
        {
            p += 4;
            return j;
        }
        return parse_number(t, p);
    }
};
} // namespace isti::host
