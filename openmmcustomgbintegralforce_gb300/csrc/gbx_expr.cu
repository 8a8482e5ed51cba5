// Expression parser, symbolic derivatives and CUDA source emission for the
// custom CharmmGBMVForce path (host code).
//
// The syntax is OpenMM's (Lepton): + - * / ^, unary minus, parentheses,
// numbers, variables and the functions below; "expr; a = ...; b = ..."
// defines intermediate values, each of which may use the ones after it.
#include <cctype>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <set>
#include <sstream>
#include <stdexcept>

#include "gbx_expr.h"

namespace gbx {
namespace expr {

namespace {

Ptr make(Op op, std::vector<Ptr> args, double value = 0.0, const std::string& name = "") {
  auto n = std::make_shared<Node>();
  n->op = op;
  n->args = std::move(args);
  n->value = value;
  n->name = name;
  return n;
}

bool is_const(const Ptr& e, double v) { return e->op == Op::Const && e->value == v; }
bool is_const(const Ptr& e) { return e->op == Op::Const; }

const std::set<std::string>& unary_functions() {
  static const std::set<std::string> f = {"sqrt", "exp",  "log",  "sin",  "cos",    "tan",   "asin",  "acos",
                                          "atan", "sinh", "cosh", "tanh", "erf",    "erfc",  "step",  "square",
                                          "cube", "recip", "abs", "floor", "ceil"};
  return f;
}

Ptr func(const std::string& name, std::vector<Ptr> args) {
  // constant folding of a function of constants
  bool all_const = true;
  for (auto& a : args) all_const = all_const && is_const(a);
  if (all_const) {
    const double x = args[0]->value;
    if (name == "sqrt") return constant(std::sqrt(x));
    if (name == "exp") return constant(std::exp(x));
    if (name == "log") return constant(std::log(x));
    if (name == "square") return constant(x * x);
    if (name == "cube") return constant(x * x * x);
    if (name == "recip") return constant(1.0 / x);
    if (name == "step") return constant(x >= 0.0 ? 1.0 : 0.0);
  }
  return make(Op::Func, std::move(args), 0.0, name);
}

Ptr add(const Ptr& a, const Ptr& b) {
  if (is_const(a, 0.0)) return b;
  if (is_const(b, 0.0)) return a;
  if (is_const(a) && is_const(b)) return constant(a->value + b->value);
  return make(Op::Add, {a, b});
}
Ptr sub(const Ptr& a, const Ptr& b) {
  if (is_const(b, 0.0)) return a;
  if (is_const(a) && is_const(b)) return constant(a->value - b->value);
  if (is_const(a, 0.0)) return make(Op::Neg, {b});
  return make(Op::Sub, {a, b});
}
Ptr mul(const Ptr& a, const Ptr& b) {
  if (is_const(a, 0.0) || is_const(b, 0.0)) return constant(0.0);
  if (is_const(a, 1.0)) return b;
  if (is_const(b, 1.0)) return a;
  if (is_const(a) && is_const(b)) return constant(a->value * b->value);
  return make(Op::Mul, {a, b});
}
Ptr div(const Ptr& a, const Ptr& b) {
  if (is_const(a, 0.0)) return constant(0.0);
  if (is_const(b, 1.0)) return a;
  if (is_const(a) && is_const(b)) return constant(a->value / b->value);
  return make(Op::Div, {a, b});
}
Ptr neg(const Ptr& a) {
  if (is_const(a)) return constant(-a->value);
  if (a->op == Op::Neg) return a->args[0];
  return make(Op::Neg, {a});
}
Ptr pw(const Ptr& a, const Ptr& b) {
  if (is_const(b, 0.0)) return constant(1.0);
  if (is_const(b, 1.0)) return a;
  if (is_const(a) && is_const(b)) return constant(std::pow(a->value, b->value));
  return make(Op::Pow, {a, b});
}

// ---------------------------------------------------------------------------
// Parser (recursive descent: sums of products of signed powers)
// ---------------------------------------------------------------------------
class Parser {
 public:
  Parser(const std::string& s, const std::set<std::string>& functions) : s_(s), functions_(functions) {}
  Ptr expression() {
    Ptr e = term();
    for (;;) {
      skip();
      if (peek('+')) {
        ++p_;
        e = add(e, term());
      } else if (peek('-')) {
        ++p_;
        e = sub(e, term());
      } else {
        return e;
      }
    }
  }
  bool at_end() {
    skip();
    return p_ >= s_.size();
  }
  std::string where() const { return "at position " + std::to_string(p_) + " of '" + s_ + "'"; }

 private:
  Ptr term() {
    Ptr e = unary();
    for (;;) {
      skip();
      if (peek('*')) {
        ++p_;
        e = mul(e, unary());
      } else if (peek('/')) {
        ++p_;
        e = div(e, unary());
      } else {
        return e;
      }
    }
  }
  Ptr unary() {
    skip();
    if (peek('-')) {
      ++p_;
      return neg(unary());
    }
    if (peek('+')) {
      ++p_;
      return unary();
    }
    return power();
  }
  Ptr power() {
    Ptr base = primary();
    skip();
    if (peek('^')) {
      ++p_;
      return pw(base, unary());  // right associative, binds a signed exponent
    }
    return base;
  }
  Ptr primary() {
    skip();
    if (p_ >= s_.size()) throw std::runtime_error("unexpected end of expression " + where());
    const char c = s_[p_];
    if (c == '(') {
      ++p_;
      Ptr e = expression();
      expect(')');
      return e;
    }
    if (std::isdigit((unsigned char)c) || c == '.') {
      const char* b = s_.c_str() + p_;
      char* end = nullptr;
      const double v = std::strtod(b, &end);
      if (end == b) throw std::runtime_error("bad number " + where());
      p_ += end - b;
      return constant(v);
    }
    if (std::isalpha((unsigned char)c) || c == '_') {
      size_t q = p_;
      while (q < s_.size() && (std::isalnum((unsigned char)s_[q]) || s_[q] == '_')) ++q;
      const std::string name = s_.substr(p_, q - p_);
      p_ = q;
      skip();
      if (peek('(')) {
        ++p_;
        std::vector<Ptr> args;
        args.push_back(expression());
        skip();
        while (peek(',')) {
          ++p_;
          args.push_back(expression());
          skip();
        }
        expect(')');
        if (functions_.count(name)) {
          if (args.size() != 1)
            throw std::runtime_error("tabulated function " + name + " takes one argument " + where());
          return make(Op::Func, std::move(args), 0.0, "@0:" + name);
        }
        const bool unary_fn = unary_functions().count(name) != 0;
        const bool binary_fn = name == "min" || name == "max";
        const bool ternary_fn = name == "select";
        if (!(unary_fn && args.size() == 1) && !(binary_fn && args.size() == 2) &&
            !(ternary_fn && args.size() == 3))
          throw std::runtime_error("unknown function or wrong argument count: " + name + " " + where());
        return func(name, std::move(args));
      }
      return variable(name);
    }
    throw std::runtime_error(std::string("unexpected character '") + c + "' " + where());
  }
  void skip() {
    while (p_ < s_.size() && std::isspace((unsigned char)s_[p_])) ++p_;
  }
  bool peek(char c) const { return p_ < s_.size() && s_[p_] == c; }
  void expect(char c) {
    skip();
    if (!peek(c)) throw std::runtime_error(std::string("expected '") + c + "' " + where());
    ++p_;
  }
  const std::string& s_;
  const std::set<std::string>& functions_;
  size_t p_ = 0;
};

Ptr substitute(const Ptr& e, const std::map<std::string, Ptr>& defs, std::set<std::string>& active) {
  if (e->op == Op::Var) {
    auto it = defs.find(e->name);
    if (it == defs.end()) return e;
    if (active.count(e->name)) throw std::runtime_error("circular definition of " + e->name);
    active.insert(e->name);
    Ptr r = substitute(it->second, defs, active);
    active.erase(e->name);
    return r;
  }
  if (e->op == Op::Const) return e;
  std::vector<Ptr> args;
  for (auto& a : e->args) args.push_back(substitute(a, defs, active));
  switch (e->op) {
    case Op::Add: return add(args[0], args[1]);
    case Op::Sub: return sub(args[0], args[1]);
    case Op::Mul: return mul(args[0], args[1]);
    case Op::Div: return div(args[0], args[1]);
    case Op::Pow: return pw(args[0], args[1]);
    case Op::Neg: return neg(args[0]);
    default: return func(e->name, args);
  }
}

std::string trim(const std::string& s) {
  size_t b = s.find_first_not_of(" \t\n\r"), e = s.find_last_not_of(" \t\n\r");
  return b == std::string::npos ? std::string() : s.substr(b, e - b + 1);
}

std::string number(double v, bool fp32) {
  char buf[64];
  std::snprintf(buf, sizeof(buf), "%.17g", v);
  std::string s = buf;
  if (s.find_first_of(".eEn") == std::string::npos) s += ".0";
  if (fp32) s += "f";
  return "(" + s + ")";
}

}  // namespace

Ptr constant(double v) { return make(Op::Const, {}, v); }
Ptr variable(const std::string& name) { return make(Op::Var, {}, 0.0, name); }

Ptr parse(const std::string& text, const std::set<std::string>& functions) {
  std::vector<std::string> parts;
  std::stringstream ss(text);
  std::string part;
  while (std::getline(ss, part, ';')) parts.push_back(part);
  if (parts.empty() || trim(parts[0]).empty()) throw std::runtime_error("empty expression");
  std::map<std::string, Ptr> defs;
  for (size_t k = 1; k < parts.size(); ++k) {
    const std::string d = trim(parts[k]);
    if (d.empty()) continue;
    const size_t eq = d.find('=');
    if (eq == std::string::npos) throw std::runtime_error("definition without '=': " + d);
    const std::string name = trim(d.substr(0, eq));
    const std::string body = d.substr(eq + 1);
    Parser p(body, functions);
    Ptr e = p.expression();
    if (!p.at_end()) throw std::runtime_error("trailing characters " + p.where());
    defs[name] = e;
  }
  Parser p(parts[0], functions);
  Ptr e = p.expression();
  if (!p.at_end()) throw std::runtime_error("trailing characters " + p.where());
  std::set<std::string> active;
  return substitute(e, defs, active);
}

void variables(const Ptr& e, std::vector<std::string>& out) {
  if (e->op == Op::Var) {
    for (auto& v : out)
      if (v == e->name) return;
    out.push_back(e->name);
    return;
  }
  for (auto& a : e->args) variables(a, out);
}

Ptr derivative(const Ptr& e, const std::string& v) {
  switch (e->op) {
    case Op::Const: return constant(0.0);
    case Op::Var: return constant(e->name == v ? 1.0 : 0.0);
    case Op::Add: return add(derivative(e->args[0], v), derivative(e->args[1], v));
    case Op::Sub: return sub(derivative(e->args[0], v), derivative(e->args[1], v));
    case Op::Neg: return neg(derivative(e->args[0], v));
    case Op::Mul: {
      const Ptr &a = e->args[0], &b = e->args[1];
      return add(mul(derivative(a, v), b), mul(a, derivative(b, v)));
    }
    case Op::Div: {
      const Ptr &a = e->args[0], &b = e->args[1];
      // (a' b - a b') / b^2
      return div(sub(mul(derivative(a, v), b), mul(a, derivative(b, v))), mul(b, b));
    }
    case Op::Pow: {
      const Ptr &a = e->args[0], &b = e->args[1];
      const Ptr da = derivative(a, v), db = derivative(b, v);
      if (is_const(db, 0.0)) return mul(mul(b, pw(a, sub(b, constant(1.0)))), da);
      // a^b (b' log a + b a' / a)
      return mul(e, add(mul(db, func("log", {a})), div(mul(b, da), a)));
    }
    case Op::Func: {
      const std::string& f = e->name;
      if (f == "min" || f == "max") {
        const Ptr &a = e->args[0], &b = e->args[1];
        // min: a where a <= b; max: a where a >= b
        const Ptr sa = f == "min" ? func("step", {sub(b, a)}) : func("step", {sub(a, b)});
        return add(mul(sa, derivative(a, v)), mul(sub(constant(1.0), sa), derivative(b, v)));
      }
      if (f == "select") return func("select", {e->args[0], derivative(e->args[1], v), derivative(e->args[2], v)});
      const Ptr& u = e->args[0];
      const Ptr du = derivative(u, v);
      if (is_const(du, 0.0)) return constant(0.0);
      Ptr g;  // d f / d u
      if (f[0] == '@') {
        // a tabulated function: its next derivative (a cubic spline has two)
        const int k = f[1] - '0';
        if (k >= 2) throw std::runtime_error("third derivative of tabulated function " + f.substr(3) + " requested");
        g = make(Op::Func, {u}, 0.0, "@" + std::to_string(k + 1) + ":" + f.substr(3));
      } else if (f == "sqrt") g = div(constant(0.5), e);
      else if (f == "exp") g = e;
      else if (f == "log") g = div(constant(1.0), u);
      else if (f == "sin") g = func("cos", {u});
      else if (f == "cos") g = neg(func("sin", {u}));
      else if (f == "tan") g = add(constant(1.0), mul(e, e));
      else if (f == "asin") g = div(constant(1.0), func("sqrt", {sub(constant(1.0), mul(u, u))}));
      else if (f == "acos") g = neg(div(constant(1.0), func("sqrt", {sub(constant(1.0), mul(u, u))})));
      else if (f == "atan") g = div(constant(1.0), add(constant(1.0), mul(u, u)));
      else if (f == "sinh") g = func("cosh", {u});
      else if (f == "cosh") g = func("sinh", {u});
      else if (f == "tanh") g = sub(constant(1.0), mul(e, e));
      else if (f == "erf") g = mul(constant(2.0 / std::sqrt(M_PI)), func("exp", {neg(mul(u, u))}));
      else if (f == "erfc") g = mul(constant(-2.0 / std::sqrt(M_PI)), func("exp", {neg(mul(u, u))}));
      else if (f == "square") g = mul(constant(2.0), u);
      else if (f == "cube") g = mul(constant(3.0), mul(u, u));
      else if (f == "recip") g = neg(div(constant(1.0), mul(u, u)));
      else if (f == "abs") g = sub(mul(constant(2.0), func("step", {u})), constant(1.0));
      else g = constant(0.0);  // step, floor, ceil: piecewise constant
      return mul(g, du);
    }
  }
  return constant(0.0);
}

std::string emit(const Ptr& e, const std::map<std::string, std::string>& rename, bool fp32) {
  const std::string f = fp32 ? "f" : "";
  switch (e->op) {
    case Op::Const: return number(e->value, fp32);
    case Op::Var: {
      auto it = rename.find(e->name);
      if (it == rename.end()) throw std::runtime_error("unknown variable in expression: " + e->name);
      return it->second;
    }
    case Op::Add: return "(" + emit(e->args[0], rename, fp32) + " + " + emit(e->args[1], rename, fp32) + ")";
    case Op::Sub: return "(" + emit(e->args[0], rename, fp32) + " - " + emit(e->args[1], rename, fp32) + ")";
    case Op::Mul: return "(" + emit(e->args[0], rename, fp32) + " * " + emit(e->args[1], rename, fp32) + ")";
    case Op::Div: return "(" + emit(e->args[0], rename, fp32) + " / " + emit(e->args[1], rename, fp32) + ")";
    case Op::Neg: return "(-" + emit(e->args[0], rename, fp32) + ")";
    case Op::Pow: {
      const std::string a = emit(e->args[0], rename, fp32);
      if (is_const(e->args[1])) {
        const double k = e->args[1]->value;
        if (k == std::floor(k) && std::fabs(k) <= 8) {  // small integer powers by multiplication
          const int m = (int)std::fabs(k);
          std::string p = "gbx_ipow" + std::to_string(m) + "(" + a + ")";
          return k < 0 ? "(" + number(1.0, fp32) + " / " + p + ")" : p;
        }
        if (k == 0.5) return "sqrt" + f + "(" + a + ")";
        if (k == 0.25) return "sqrt" + f + "(sqrt" + f + "(" + a + "))";
      }
      return "pow" + f + "(" + a + ", " + emit(e->args[1], rename, fp32) + ")";
    }
    case Op::Func: {
      std::vector<std::string> a;
      for (auto& x : e->args) a.push_back(emit(x, rename, fp32));
      const std::string& n = e->name;
      if (n[0] == '@') return "gbx_tab_" + n.substr(3) + "_" + n.substr(1, 1) + "(" + a[0] + ")";
      if (n == "step") return "((" + a[0] + ") >= 0 ? " + number(1.0, fp32) + " : " + number(0.0, fp32) + ")";
      if (n == "square") return "gbx_ipow2(" + a[0] + ")";
      if (n == "cube") return "gbx_ipow3(" + a[0] + ")";
      if (n == "recip") return "(" + number(1.0, fp32) + " / " + a[0] + ")";
      if (n == "abs") return "fabs" + f + "(" + a[0] + ")";
      if (n == "min") return "fmin" + f + "(" + a[0] + ", " + a[1] + ")";
      if (n == "max") return "fmax" + f + "(" + a[0] + ", " + a[1] + ")";
      if (n == "select") return "((" + a[0] + ") != 0 ? " + a[1] + " : " + a[2] + ")";
      return n + f + "(" + a[0] + ")";
    }
  }
  return number(0.0, fp32);
}

SharedEmitter::SharedEmitter(const std::map<std::string, std::string>& rename, bool fp32, std::string prefix,
                             std::string indent)
    : rename_(rename), fp32_(fp32), prefix_(std::move(prefix)), indent_(std::move(indent)) {}

std::string SharedEmitter::take_decls() {
  std::string d;
  d.swap(decls_);
  return d;
}

std::string SharedEmitter::operator()(const Ptr& e) { return node(e); }

std::string SharedEmitter::intern(const std::string& text) {
  auto same = by_text_.find(text);
  if (same != by_text_.end()) return same->second;
  const std::string name = prefix_ + std::to_string(by_text_.size());
  by_text_[text] = name;
  decls_ += indent_ + "const " + (fp32_ ? "float " : "double ") + name + " = " + text + ";\n";
  return name;
}

std::string SharedEmitter::node(const Ptr& e) {
  if (e->op == Op::Const || e->op == Op::Var) return emit(e, rename_, fp32_);
  auto hit = by_node_.find(e.get());
  if (hit != by_node_.end()) return hit->second;
  // the node's text over its children's names
  std::vector<std::string> a;
  for (auto& x : e->args) a.push_back(node(x));
  if (fp32_ && e->op == Op::Div && e->args[1]->op != Op::Const) {
    // FP32 quotients share one reciprocal per denominator (the generated
    // FP32 code is compiled with fast math, where a quotient is a
    // reciprocal and a product anyway)
    // 1 / (x x) as the square of 1 / x (one reciprocal serves both)
    const Ptr& den = e->args[1];
    std::string r;
    if (den->op == Op::Mul && den->args[0]->op != Op::Const && node(den->args[0]) == node(den->args[1])) {
      const std::string rx = intern("(1.0f / " + node(den->args[0]) + ")");
      r = intern("(" + rx + " * " + rx + ")");
    } else {
      r = intern("(1.0f / " + a[1] + ")");
    }
    const bool one = e->args[0]->op == Op::Const && e->args[0]->value == 1.0;
    const std::string name = one ? r : intern("(" + a[0] + " * " + r + ")");
    by_node_[e.get()] = name;
    keep_.push_back(e);
    return name;
  }
  std::vector<Ptr> leaves;
  for (size_t k = 0; k < a.size(); ++k) leaves.push_back(variable("\x01" + std::to_string(k)));
  std::map<std::string, std::string> rn;
  for (size_t k = 0; k < a.size(); ++k) rn["\x01" + std::to_string(k)] = a[k];
  Node shell = *e;
  shell.args.clear();
  for (size_t k = 0; k < e->args.size(); ++k)
    shell.args.push_back(e->args[k]->op == Op::Const ? e->args[k] : leaves[k]);
  const std::string name = intern(emit(std::make_shared<const Node>(shell), rn, fp32_));
  by_node_[e.get()] = name;
  keep_.push_back(e);
  return name;
}

}  // namespace expr
}  // namespace gbx
