// json.hh -- DiFfRG::JSONValue without boost::json: the parameter object that generated flow
// classes and the integrator constructors take (DiFfRG/include/DiFfRG/common/json.hh:18-189 --
// same class name, same get_/set_ accessors with '/'-separated paths, same defaults overloads).
//
// A value is null, a bool, a number, a string, an array or an object (key order kept).  The
// constructor taking a std::string reads that file, as the reference's does; a string whose first
// non-blank character is '{' is parsed as JSON text instead (in place of the reference's
// boost::json::value constructor, which has no counterpart without boost).  Lookups of a missing
// key throw std::runtime_error naming the path; numbers convert between int/uint/double on
// access, as boost::json's to_number does.  Host code only.
#pragma once

#include <cctype>
#include <cmath>
#include <cstdlib>
#include <fstream>
#include <map>
#include <memory>
#include <ostream>
#include <sstream>
#include <stdexcept>
#include <string>
#include <utility>
#include <vector>

namespace DiFfRG
{
  namespace gbint_json
  {
    struct Node {
      enum Kind { Null, Bool, Number, String, Array, Object } kind = Null;
      bool b = false;
      double num = 0;
      bool integral = false;  // written without fraction/exponent: printed back as an integer
      std::string str;
      std::vector<Node> arr;
      std::vector<std::pair<std::string, Node>> obj;

      Node *find(const std::string &k)
      {
        for (auto &kv : obj)
          if (kv.first == k) return &kv.second;
        return nullptr;
      }
      const Node *find(const std::string &k) const { return const_cast<Node *>(this)->find(k); }
      bool operator==(const Node &o) const
      {
        if (kind != o.kind) return false;
        switch (kind) {
        case Null: return true;
        case Bool: return b == o.b;
        case Number: return num == o.num;
        case String: return str == o.str;
        case Array: return arr == o.arr;
        case Object: {
          if (obj.size() != o.obj.size()) return false;
          for (const auto &kv : obj) {
            const Node *p = o.find(kv.first);
            if (!p || !(*p == kv.second)) return false;
          }
          return true;
        }
        }
        return false;
      }
    };

    class Parser
    {
    public:
      explicit Parser(const std::string &s) : s_(s) {}
      Node parse()
      {
        Node n = value();
        ws();
        if (i_ != s_.size()) fail("trailing characters");
        return n;
      }

    private:
      [[noreturn]] void fail(const char *what) const
      {
        throw std::runtime_error(std::string("JSONValue: ") + what + " at offset " + std::to_string(i_));
      }
      void ws()
      {
        while (i_ < s_.size() && std::isspace((unsigned char)s_[i_])) ++i_;
      }
      bool eat(char c)
      {
        ws();
        if (i_ < s_.size() && s_[i_] == c) {
          ++i_;
          return true;
        }
        return false;
      }
      void expect(char c)
      {
        if (!eat(c)) fail((std::string("expected '") + c + "'").c_str());
      }
      bool word(const char *w)
      {
        const std::string t(w);
        if (s_.compare(i_, t.size(), t) == 0) {
          i_ += t.size();
          return true;
        }
        return false;
      }
      static void utf8(std::string &o, unsigned cp)
      {
        if (cp < 0x80)
          o += (char)cp;
        else if (cp < 0x800) {
          o += (char)(0xC0 | (cp >> 6));
          o += (char)(0x80 | (cp & 0x3F));
        } else if (cp < 0x10000) {
          o += (char)(0xE0 | (cp >> 12));
          o += (char)(0x80 | ((cp >> 6) & 0x3F));
          o += (char)(0x80 | (cp & 0x3F));
        } else {
          o += (char)(0xF0 | (cp >> 18));
          o += (char)(0x80 | ((cp >> 12) & 0x3F));
          o += (char)(0x80 | ((cp >> 6) & 0x3F));
          o += (char)(0x80 | (cp & 0x3F));
        }
      }
      unsigned hex4()
      {
        if (i_ + 4 > s_.size()) fail("short \\u escape");
        unsigned v = 0;
        for (int k = 0; k < 4; ++k) {
          const char c = s_[i_++];
          v <<= 4;
          if (c >= '0' && c <= '9')
            v |= (unsigned)(c - '0');
          else if (c >= 'a' && c <= 'f')
            v |= (unsigned)(c - 'a' + 10);
          else if (c >= 'A' && c <= 'F')
            v |= (unsigned)(c - 'A' + 10);
          else
            fail("bad \\u escape");
        }
        return v;
      }
      std::string string_body()
      {
        std::string o;
        for (;;) {
          if (i_ >= s_.size()) fail("unterminated string");
          const char c = s_[i_++];
          if (c == '"') return o;
          if (c != '\\') {
            o += c;
            continue;
          }
          if (i_ >= s_.size()) fail("unterminated escape");
          const char e = s_[i_++];
          switch (e) {
          case '"': o += '"'; break;
          case '\\': o += '\\'; break;
          case '/': o += '/'; break;
          case 'b': o += '\b'; break;
          case 'f': o += '\f'; break;
          case 'n': o += '\n'; break;
          case 'r': o += '\r'; break;
          case 't': o += '\t'; break;
          case 'u': {
            unsigned cp = hex4();
            if (cp >= 0xD800 && cp < 0xDC00 && i_ + 1 < s_.size() && s_[i_] == '\\' && s_[i_ + 1] == 'u') {
              i_ += 2;
              const unsigned lo = hex4();
              cp = 0x10000 + ((cp - 0xD800) << 10) + (lo - 0xDC00);
            }
            utf8(o, cp);
            break;
          }
          default: fail("bad escape");
          }
        }
      }
      Node value()
      {
        ws();
        if (i_ >= s_.size()) fail("unexpected end");
        Node n;
        const char c = s_[i_];
        if (c == '{') {
          ++i_;
          n.kind = Node::Object;
          if (eat('}')) return n;
          do {
            ws();
            expect('"');
            std::string k = string_body();
            expect(':');
            Node v = value();
            if (Node *old = n.find(k))
              *old = std::move(v);  // a repeated key keeps the last value
            else
              n.obj.emplace_back(std::move(k), std::move(v));
          } while (eat(','));
          expect('}');
        } else if (c == '[') {
          ++i_;
          n.kind = Node::Array;
          if (eat(']')) return n;
          do n.arr.push_back(value());
          while (eat(','));
          expect(']');
        } else if (c == '"') {
          ++i_;
          n.kind = Node::String;
          n.str = string_body();
        } else if (word("true")) {
          n.kind = Node::Bool;
          n.b = true;
        } else if (word("false")) {
          n.kind = Node::Bool;
        } else if (word("null")) {
          n.kind = Node::Null;
        } else {
          const char *b = s_.c_str() + i_;
          char *e = nullptr;
          n.num = std::strtod(b, &e);
          if (e == b) fail("bad value");
          n.kind = Node::Number;
          n.integral = true;
          for (const char *p = b; p < e; ++p)
            if (*p == '.' || *p == 'e' || *p == 'E') n.integral = false;
          i_ += (size_t)(e - b);
        }
        return n;
      }

      const std::string &s_;
      size_t i_ = 0;
    };

    inline std::vector<std::string> split_path(const std::string &key)
    {
      std::vector<std::string> parts;
      std::string cur;
      for (char c : key) {
        if (c == '/') {
          if (!cur.empty()) parts.push_back(cur);
          cur.clear();
        } else
          cur += c;
      }
      if (!cur.empty()) parts.push_back(cur);
      return parts;
    }

    inline void write_string(std::ostream &os, const std::string &s)
    {
      os << '"';
      for (char c : s) {
        switch (c) {
        case '"': os << "\\\""; break;
        case '\\': os << "\\\\"; break;
        case '\n': os << "\\n"; break;
        case '\t': os << "\\t"; break;
        case '\r': os << "\\r"; break;
        default: os << c;
        }
      }
      os << '"';
    }

    inline void write(std::ostream &os, const Node &n, int indent, int level)
    {
      const std::string pad = indent ? std::string((size_t)indent * (level + 1), ' ') : std::string();
      const std::string end = indent ? std::string((size_t)indent * level, ' ') : std::string();
      const char *nl = indent ? "\n" : "";
      switch (n.kind) {
      case Node::Null: os << "null"; break;
      case Node::Bool: os << (n.b ? "true" : "false"); break;
      case Node::Number:
        if (n.integral && std::fabs(n.num) < 9.0e15)
          os << (long long)n.num;
        else {
          std::ostringstream t;
          t.precision(17);
          t << n.num;
          os << t.str();
        }
        break;
      case Node::String: write_string(os, n.str); break;
      case Node::Array:
        os << '[' << nl;
        for (size_t i = 0; i < n.arr.size(); ++i) {
          os << pad;
          write(os, n.arr[i], indent, level + 1);
          os << (i + 1 < n.arr.size() ? "," : "") << nl;
        }
        os << end << ']';
        break;
      case Node::Object:
        os << '{' << nl;
        for (size_t i = 0; i < n.obj.size(); ++i) {
          os << pad;
          write_string(os, n.obj[i].first);
          os << (indent ? ": " : ":");
          write(os, n.obj[i].second, indent, level + 1);
          os << (i + 1 < n.obj.size() ? "," : "") << nl;
        }
        os << end << '}';
        break;
      }
    }
  } // namespace gbint_json

  class JSONValue
  {
  public:
    using uint = unsigned int;
    JSONValue() : root_(std::make_shared<gbint_json::Node>()) { root_->kind = gbint_json::Node::Object; }
    // a file name (the reference's constructor), or JSON text starting with '{'
    JSONValue(const std::string filename_or_text) : JSONValue()
    {
      size_t p = 0;
      while (p < filename_or_text.size() && std::isspace((unsigned char)filename_or_text[p])) ++p;
      if (p < filename_or_text.size() && filename_or_text[p] == '{') {
        *root_ = gbint_json::Parser(filename_or_text).parse();
        return;
      }
      std::ifstream f(filename_or_text);
      if (!f) throw std::runtime_error("JSONValue: could not open file " + filename_or_text);
      std::stringstream ss;
      ss << f.rdbuf();
      const std::string text = ss.str();
      *root_ = gbint_json::Parser(text).parse();
    }
    JSONValue(const char *filename_or_text) : JSONValue(std::string(filename_or_text)) {}
    // copies are deep, as copies of a boost::json::value are
    JSONValue(const JSONValue &o) : root_(std::make_shared<gbint_json::Node>(*o.root_)) {}
    JSONValue &operator=(const JSONValue &o)
    {
      if (this != &o) root_ = std::make_shared<gbint_json::Node>(*o.root_);
      return *this;
    }

    bool operator==(const JSONValue &other) const { return *root_ == *other.root_; }

    double get_double(const std::string &key) const { return number(key); }
    int get_int(const std::string &key) const { return (int)std::llround(number(key)); }
    uint get_uint(const std::string &key) const
    {
      const double v = number(key);
      if (v < 0) throw std::runtime_error("JSONValue: " + key + " is negative, expected an unsigned value");
      return (uint)std::llround(v);
    }
    std::string get_string(const std::string &key) const
    {
      const gbint_json::Node &n = at(key);
      if (n.kind != gbint_json::Node::String) throw std::runtime_error("JSONValue: " + key + " is not a string");
      return n.str;
    }
    bool get_bool(const std::string &key) const
    {
      const gbint_json::Node &n = at(key);
      if (n.kind == gbint_json::Node::Bool) return n.b;
      if (n.kind == gbint_json::Node::Number) return n.num != 0;
      throw std::runtime_error("JSONValue: " + key + " is not a bool");
    }

    double get_double(const std::string &key, const double def) const { return has(key) ? get_double(key) : def; }
    int get_int(const std::string &key, const int def) const { return has(key) ? get_int(key) : def; }
    uint get_uint(const std::string &key, const uint def) const { return has(key) ? get_uint(key) : def; }
    std::string get_string(const std::string &key, const std::string &def) const
    {
      return has(key) ? get_string(key) : def;
    }
    bool get_bool(const std::string &key, const bool def) const { return has(key) ? get_bool(key) : def; }

    void set_double(const std::string &key, double value) { set_number(key, value, false); }
    void set_int(const std::string &key, int value) { set_number(key, (double)value, true); }
    void set_uint(const std::string &key, uint value) { set_number(key, (double)value, true); }
    void set_string(const std::string &key, const std::string &value)
    {
      gbint_json::Node &n = make(key);
      n = gbint_json::Node();
      n.kind = gbint_json::Node::String;
      n.str = value;
    }
    void set_bool(const std::string &key, bool value)
    {
      gbint_json::Node &n = make(key);
      n = gbint_json::Node();
      n.kind = gbint_json::Node::Bool;
      n.b = value;
    }

    // true when the path names an existing entry (no counterpart in the reference)
    bool has(const std::string &key) const { return lookup(key) != nullptr; }

    void print(std::ostream &os) const
    {
      gbint_json::write(os, *root_, 2, 0);
      os << "\n";
    }
    std::string dump() const
    {
      std::ostringstream os;
      gbint_json::write(os, *root_, 0, 0);
      return os.str();
    }

  private:
    const gbint_json::Node *lookup(const std::string &key) const
    {
      const gbint_json::Node *n = root_.get();
      for (const auto &p : gbint_json::split_path(key)) {
        if (n->kind == gbint_json::Node::Object)
          n = n->find(p);
        else if (n->kind == gbint_json::Node::Array) {
          char *e = nullptr;
          const long i = std::strtol(p.c_str(), &e, 10);
          n = (*e == 0 && i >= 0 && (size_t)i < n->arr.size()) ? &n->arr[(size_t)i] : nullptr;
        } else
          n = nullptr;
        if (!n) return nullptr;
      }
      return n;
    }
    const gbint_json::Node &at(const std::string &key) const
    {
      const gbint_json::Node *n = lookup(key);
      if (!n) throw std::runtime_error("JSONValue: no entry " + key);
      return *n;
    }
    double number(const std::string &key) const
    {
      const gbint_json::Node &n = at(key);
      if (n.kind == gbint_json::Node::Number) return n.num;
      if (n.kind == gbint_json::Node::Bool) return n.b ? 1.0 : 0.0;
      throw std::runtime_error("JSONValue: " + key + " is not a number");
    }
    gbint_json::Node &make(const std::string &key)
    {
      gbint_json::Node *n = root_.get();
      for (const auto &p : gbint_json::split_path(key)) {
        if (n->kind != gbint_json::Node::Object) {
          *n = gbint_json::Node();
          n->kind = gbint_json::Node::Object;
        }
        gbint_json::Node *c = n->find(p);
        if (!c) {
          n->obj.emplace_back(p, gbint_json::Node());
          c = &n->obj.back().second;
        }
        n = c;
      }
      return *n;
    }
    void set_number(const std::string &key, double v, bool integral)
    {
      gbint_json::Node &n = make(key);
      n = gbint_json::Node();
      n.kind = gbint_json::Node::Number;
      n.num = v;
      n.integral = integral;
    }

    std::shared_ptr<gbint_json::Node> root_;
  };
} // namespace DiFfRG
