// json.hpp -- a small JSON reader for Galaxy's state files (the role
// rapidjson plays in the Galaxy tree: Camera::LoadFromJSON, Lighting::
// LoadStateFromValue, Visualization::LoadFromJSON, Datasets::LoadFromJSON).
// Objects keep their members in file order; numbers are doubles.
#pragma once

#include <cstdlib>
#include <map>
#include <memory>
#include <stdexcept>
#include <string>
#include <utility>
#include <vector>

namespace gxyhost {

class Json {
  public:
    enum Kind { Null, Bool, Number, String, Array, Object };

    Json() = default;
    Kind kind() const { return kind_; }
    bool is_object() const { return kind_ == Object; }
    bool is_array() const { return kind_ == Array; }
    bool is_string() const { return kind_ == String; }
    bool is_number() const { return kind_ == Number; }
    bool is_bool() const { return kind_ == Bool; }

    bool has(const std::string &k) const {
        if (kind_ != Object) return false;
        for (auto &m : members_)
            if (m.first == k) return true;
        return false;
    }
    const Json &operator[](const std::string &k) const {
        if (kind_ != Object) throw std::runtime_error("json: not an object (looking for \"" + k + "\")");
        for (auto &m : members_)
            if (m.first == k) return m.second;
        throw std::runtime_error("json: no member \"" + k + "\"");
    }
    const Json &operator[](size_t i) const {
        if (kind_ != Array || i >= items_.size()) throw std::runtime_error("json: bad array index");
        return items_[i];
    }
    size_t size() const { return kind_ == Array ? items_.size() : kind_ == Object ? members_.size() : 0; }
    double num() const {
        if (kind_ == Bool) return b_ ? 1.0 : 0.0;
        if (kind_ != Number) throw std::runtime_error("json: not a number");
        return n_;
    }
    bool boolean() const {
        if (kind_ == Number) return n_ != 0.0;
        if (kind_ != Bool) throw std::runtime_error("json: not a boolean");
        return b_;
    }
    const std::string &str() const {
        if (kind_ != String) throw std::runtime_error("json: not a string");
        return s_;
    }
    const std::vector<std::pair<std::string, Json>> &members() const { return members_; }

    static Json parse(const std::string &text) {
        size_t p = 0;
        Json v = value(text, p);
        ws(text, p);
        if (p != text.size()) throw std::runtime_error("json: trailing characters");
        return v;
    }

  private:
    Kind kind_ = Null;
    bool b_ = false;
    double n_ = 0.0;
    std::string s_;
    std::vector<Json> items_;
    std::vector<std::pair<std::string, Json>> members_;

    static void ws(const std::string &t, size_t &p) {
        while (p < t.size() && (t[p] == ' ' || t[p] == '\t' || t[p] == '\n' || t[p] == '\r')) p++;
    }
    static void expect(const std::string &t, size_t &p, char c) {
        ws(t, p);
        if (p >= t.size() || t[p] != c) throw std::runtime_error(std::string("json: expected '") + c + "'");
        p++;
    }
    static std::string string_(const std::string &t, size_t &p) {
        expect(t, p, '"');
        std::string out;
        while (p < t.size() && t[p] != '"') {
            char c = t[p++];
            if (c == '\\') {
                if (p >= t.size()) break;
                char e = t[p++];
                switch (e) {
                    case 'n': out += '\n'; break;
                    case 't': out += '\t'; break;
                    case 'r': out += '\r'; break;
                    case 'b': out += '\b'; break;
                    case 'f': out += '\f'; break;
                    case 'u': {   // \uXXXX, kept as UTF-8 for the basic plane
                        if (p + 4 > t.size()) throw std::runtime_error("json: bad escape");
                        unsigned cp = (unsigned)std::strtoul(t.substr(p, 4).c_str(), nullptr, 16);
                        p += 4;
                        if (cp < 0x80) out += (char)cp;
                        else if (cp < 0x800) {
                            out += (char)(0xc0 | (cp >> 6));
                            out += (char)(0x80 | (cp & 0x3f));
                        } else {
                            out += (char)(0xe0 | (cp >> 12));
                            out += (char)(0x80 | ((cp >> 6) & 0x3f));
                            out += (char)(0x80 | (cp & 0x3f));
                        }
                        break;
                    }
                    default: out += e;
                }
            } else {
                out += c;
            }
        }
        if (p >= t.size()) throw std::runtime_error("json: unterminated string");
        p++;
        return out;
    }
    static Json value(const std::string &t, size_t &p) {
        ws(t, p);
        if (p >= t.size()) throw std::runtime_error("json: unexpected end");
        Json v;
        char c = t[p];
        if (c == '{') {
            p++;
            v.kind_ = Object;
            ws(t, p);
            if (p < t.size() && t[p] == '}') {
                p++;
                return v;
            }
            for (;;) {
                std::string k = string_(t, p);
                expect(t, p, ':');
                v.members_.emplace_back(k, value(t, p));
                ws(t, p);
                if (p < t.size() && t[p] == ',') {
                    p++;
                    continue;
                }
                expect(t, p, '}');
                return v;
            }
        }
        if (c == '[') {
            p++;
            v.kind_ = Array;
            ws(t, p);
            if (p < t.size() && t[p] == ']') {
                p++;
                return v;
            }
            for (;;) {
                v.items_.push_back(value(t, p));
                ws(t, p);
                if (p < t.size() && t[p] == ',') {
                    p++;
                    continue;
                }
                expect(t, p, ']');
                return v;
            }
        }
        if (c == '"') {
            v.kind_ = String;
            v.s_ = string_(t, p);
            return v;
        }
        if (t.compare(p, 4, "true") == 0) {
            p += 4;
            v.kind_ = Bool;
            v.b_ = true;
            return v;
        }
        if (t.compare(p, 5, "false") == 0) {
            p += 5;
            v.kind_ = Bool;
            return v;
        }
        if (t.compare(p, 4, "null") == 0) {
            p += 4;
            return v;
        }
        char *end = nullptr;
        v.n_ = std::strtod(t.c_str() + p, &end);
        if (end == t.c_str() + p) throw std::runtime_error("json: bad value");
        p = (size_t)(end - t.c_str());
        v.kind_ = Number;
        return v;
    }
};

}  // namespace gxyhost
