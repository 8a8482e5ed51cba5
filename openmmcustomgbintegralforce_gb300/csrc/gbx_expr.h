// Expressions of a CharmmGBMVForce outside the canonical CHARMM set: a
// parser for OpenMM's (Lepton) expression syntax, symbolic derivatives and
// CUDA source emission.  Host code only.
#pragma once

#include <map>
#include <memory>
#include <set>
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
// substituted, later ones may use earlier ones).  `functions` names the
// force's tabulated functions of one variable; a call f(u) becomes a node
// Op::Func named "@0:f" ("@k:f" is its k-th derivative).  Throws
// std::runtime_error with a message on a syntax error or an unknown
// function.
Ptr parse(const std::string& text, const std::set<std::string>& functions = {});

Ptr constant(double v);
Ptr variable(const std::string& name);

// d e / d var, simplified (constants folded, 0 and 1 absorbed).
Ptr derivative(const Ptr& e, const std::string& var);

// Every variable name the expression reads.
void variables(const Ptr& e, std::vector<std::string>& out);

// C source of the expression; every variable is rendered through `rename`
// (a name missing from it throws).  `fp32` selects float literals and the
// float forms of the math functions.  A tabulated function's k-th
// derivative "@k:f" is the call gbx_tab_f_k(u), which the generated source
// defines in FP64 and FP32.
std::string emit(const Ptr& e, const std::map<std::string, std::string>& rename, bool fp32);

// Emits several expressions with their common subexpressions formed once:
// the first time a node's text appears it becomes a temporary
// "const T <prefix><k> = ...;" appended to the pending declarations, and
// later uses name the temporary.  take_decls() hands the pending
// declarations to the caller, who writes them before the code that uses the
// returned names (so expressions emitted later may reuse earlier ones).
class SharedEmitter {
 public:
  SharedEmitter(const std::map<std::string, std::string>& rename, bool fp32, std::string prefix,
                std::string indent);
  std::string operator()(const Ptr& e);
  std::string take_decls();

 private:
  std::string node(const Ptr& e);
  std::string intern(const std::string& text);  // the temporary holding `text`, declared on first use
  const std::map<std::string, std::string>& rename_;
  bool fp32_;
  std::string prefix_, indent_, decls_;
  std::map<const Node*, std::string> by_node_;
  std::map<std::string, std::string> by_text_;
  std::vector<Ptr> keep_;  // nodes whose address keys by_node_
};

}  // namespace expr
}  // namespace gbx
