// Numbers in scene files: the reference reads them through its expression
// evaluator (Expr.h, Expr.cpp, used through the atof / atoi macros and the
// sscanf*f helpers of scene_env.h:24-120), so a value may be an expression
// over VAR variables.  This is a restatement of that evaluator's rules:
//
//   expr   := term { ('+' | '-') term }
//   term   := factor { ('*' | '/' | '%') factor }      a % b = a - floor(a/b)*b
//   factor := signed [ '^' factor ]                     right-associative pow
//   signed := { '-' | '+' } atom
//   atom   := literal | '(' expr ')' | constant | function '(' ... ')' | variable
//
// Blanks are skipped before an operand (and inside parentheses before '(' /
// ')' / ','), never before an operator, so "1 -2 3" and "1 - 2 3" are both
// the three values 1, -2, 3: that is how a line of several values splits.
// Literals accumulate every digit, integer and fraction, into one double
// and divide once by the base power of the fraction digits; a leading '0'
// selects the base (0x hex, 0t decimal, 0b<n>: base n, '0.' decimal, else
// octal) and an exponent multiplies or divides by base^n formed by
// repeated squaring.  Built-ins: pi, e, sqrt, exp, log, pow, sin, cos, tan,
// asin, acos, atan, atan2, sind, cosd, tand (degrees in), dasin, dacos,
// datan, datan2 (degrees out), floor, ceil.  A variable name is letters
// then letters or digits; when a name is defined twice the first value
// holds (the reference searches its list from the front).
#pragma once

#include <algorithm>
#include <cctype>
#include <cmath>
#include <cstdlib>
#include <stdexcept>
#include <string>
#include <utility>
#include <vector>

namespace pr {

class ExprError : public std::runtime_error {
 public:
  using std::runtime_error::runtime_error;
};

class ExprReader {
 public:
  void define(const std::string& name, double value) { vars_.emplace_back(name, value); }

  // one value on the whole text (the atof / atoi form).  A text that
  // starts with %NAME% is the environment variable NAME read as a value,
  // 0 when it is not set (Expr.cpp:78-110).
  double one(const std::string& text) {
    start(text);
    if (*s_ == '%') {
      const size_t e = text_.find('%', 1);
      if (e == std::string::npos || e > 80) fail("an environment reference needs a closing '%'");
      const char* v = std::getenv(text_.substr(1, e - 1).c_str());
      return v ? one(v) : 0.0;
    }
    const double x = expr();
    finish();
    return x;
  }

  // n values in a row (the sscanf*f forms)
  std::vector<double> many(const std::string& text, int n) {
    start(text);
    std::vector<double> v;
    for (int i = 0; i < n; i++) v.push_back(expr());
    finish();
    return v;
  }

 private:
  static constexpr double kPi = 3.14159265358979323846;
  std::vector<std::pair<std::string, double>> vars_;
  std::string text_;
  const char* s_ = nullptr;

  void start(const std::string& text) {
    // trailing blanks and line ends are dropped (the reference stops at a
    // trailing blank with an error instead)
    size_t e = text.size();
    while (e > 0 && std::isspace((unsigned char)text[e - 1])) e--;
    text_ = text.substr(0, e);
    s_ = text_.c_str();
  }
  void finish() {
    if (*s_) fail("unexpected text");
  }
  [[noreturn]] void fail(const char* why) {
    throw ExprError(std::string(why) + " at column " + std::to_string(s_ - text_.c_str() + 1) + " of '" + text_ + "'");
  }
  void blanks() {
    while (std::isspace((unsigned char)*s_)) s_++;
  }

  double expr() {
    blanks();
    double x = term();
    for (;;) {
      if (*s_ == '+') {
        s_++;
        x += term();
      } else if (*s_ == '-') {
        s_++;
        x -= term();
      } else {
        return x;
      }
    }
  }
  double term() {
    double x = factor();
    for (;;) {
      if (*s_ == '*') {
        s_++;
        x *= factor();
      } else if (*s_ == '/') {
        s_++;
        x /= factor();
      } else if (*s_ == '%') {
        s_++;
        const double y = factor();
        x = x - std::floor(x / y) * y;
      } else {
        return x;
      }
    }
  }
  double factor() {
    const double x = signed_atom();
    if (*s_ == '^') {
      s_++;
      return std::pow(x, factor());
    }
    return x;
  }
  double signed_atom() {
    blanks();
    if (*s_ == '-') {
      s_++;
      return -signed_atom();
    }
    if (*s_ == '+') {
      s_++;
      return signed_atom();
    }
    return atom();
  }
  double paren() {
    blanks();
    if (*s_ != '(') fail("expected '('");
    s_++;
    const double x = expr();
    blanks();
    if (*s_ != ')') fail("expected ')'");
    s_++;
    return x;
  }
  void paren2(double& x, double& y) {
    blanks();
    if (*s_ != '(') fail("expected '('");
    s_++;
    x = expr();
    blanks();
    if (*s_ != ',') fail("expected ','");
    s_++;
    y = expr();
    blanks();
    if (*s_ != ')') fail("expected ')'");
    s_++;
  }
  double atom() {
    blanks();
    if (std::isdigit((unsigned char)*s_) || *s_ == '.') return literal();
    if (*s_ == '(') return paren();
    if (!std::isalpha((unsigned char)*s_)) fail("expected a number");
    const char* b = s_;
    for (s_++; std::isalnum((unsigned char)*s_); s_++) {
    }
    const std::string n(b, s_);
    const double d2r = kPi / 180.0, r2d = 180.0 / kPi;
    double x, y;
    if (n == "pi") return kPi;
    if (n == "e") return std::exp(1.0);
    if (n == "sqrt") return std::sqrt(paren());
    if (n == "exp") return std::exp(paren());
    if (n == "log") return std::log(paren());
    if (n == "pow") {
      paren2(x, y);
      return std::pow(x, y);
    }
    if (n == "sin") return std::sin(paren());
    if (n == "cos") return std::cos(paren());
    if (n == "tan") return std::tan(paren());
    if (n == "asin") return std::asin(paren());
    if (n == "acos") return std::acos(paren());
    if (n == "atan") return std::atan(paren());
    if (n == "atan2") {
      paren2(x, y);
      return std::atan2(x, y);
    }
    if (n == "sind") return std::sin(paren() * d2r);
    if (n == "cosd") return std::cos(paren() * d2r);
    if (n == "tand") return std::tan(paren() * d2r);
    if (n == "dasin") return std::asin(paren()) * r2d;
    if (n == "dacos") return std::acos(paren()) * r2d;
    if (n == "datan") return std::atan(paren()) * r2d;
    if (n == "datan2") {
      paren2(x, y);
      return std::atan2(x, y) * r2d;
    }
    if (n == "floor") return std::floor(paren());
    if (n == "ceil") return std::ceil(paren());
    for (const auto& v : vars_)
      if (v.first == n) return v.second;
    s_ = b;
    fail(("unknown name '" + n + "'").c_str());
  }
  static int digit(int c) {
    if (c >= '0' && c <= '9') return c - '0';
    if (c >= 'a' && c <= 'z') return c - 'a' + 10;
    if (c >= 'A' && c <= 'Z') return c - 'A' + 10;
    return -1;
  }
  static double power_of(int base, int n) {
    double t = base, x = 1.0;
    for (; n > 0; n >>= 1) {
      if (n & 1) x *= t;
      t *= t;
    }
    return x;
  }
  double literal() {
    int base = 10;
    if (*s_ == '0') {
      s_++;
      if (*s_ == 'b') {
        s_++;
        for (base = 0; std::isdigit((unsigned char)*s_); s_++) base = std::min(base * 10 + (*s_ - '0'), 1000);
        if (*s_ != ':') fail("expected ':' after a base");
        s_++;
      } else if (*s_ == 'x') {
        s_++;
        base = 16;
      } else if (*s_ == 't') {
        s_++;
        base = 10;
      } else if (*s_ == '.') {
        base = 10;
      } else {
        base = 8;
      }
    }
    double x = 0.0;
    int d;
    for (; d = digit(*s_), d >= 0 && d < base; s_++) x = x * base + d;
    if (*s_ == '.') {
      s_++;
      double y = 1.0;
      for (; d = digit(*s_), d >= 0 && d < base; s_++) {
        x = x * base + d;
        y *= base;
      }
      x /= y;
    }
    if (*s_ == 'e' || *s_ == 'E') {
      s_++;
      bool up = true;
      if (*s_ == '-') {
        s_++;
        up = false;
      } else if (*s_ == '+') {
        s_++;
      }
      int n = 0;
      for (; std::isdigit((unsigned char)*s_); s_++) n = std::min(n * 10 + (*s_ - '0'), 1 << 20);
      const double y = power_of(base, n);
      if (up)
        x *= y;
      else
        x /= y;
    }
    return x;
  }
};

}  // namespace pr
