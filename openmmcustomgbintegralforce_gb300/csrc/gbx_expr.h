// Expressions of a CharmmGBMVForce outside the canonical CHARMM set: a
// parser for OpenMM's (Lepton) expression syntax, symbolic derivatives and
// CUDA source emission.  Host code only.
#pragma once

#include <map>
#include <memory>
#include <string>
#include <vector>

namespace gbx {
namespace expr {

struct Node;
using Ptr = std::shared_ptr<const Node>;

enum class Op { Const, Var, Add, Sub, Mul, Div, Pow, Neg, Func };

struct Node {
  Op op;
  double value = 0.0;  // Const
  std::string name;    // Var: variable; Func: function name
  std::vector<Ptr> args;
};

// Parses "expr" or "expr; name1 = def1; name2 = def2 ..." (definitions are
// substituted, later ones may use earlier ones).  Throws std::runtime_error
// with a message on a syntax error or an unknown function.
Ptr parse(const std::string& text);

Ptr constant(double v);
Ptr variable(const std::string& name);

// d e / d var, simplified (constants folded, 0 and 1 absorbed).
Ptr derivative(const Ptr& e, const std::string& var);

// Every variable name the expression reads.
void variables(const Ptr& e, std::vector<std::string>& out);

// C source of the expression; every variable is rendered through `rename`
// (a name missing from it throws).  `fp32` selects float literals and the
// float forms of the math functions.
std::string emit(const Ptr& e, const std::map<std::string, std::string>& rename, bool fp32);

}  // namespace expr
}  // namespace gbx
