// shl_expr.h -- the arithmetic-expression language of the config file.
//
// The reference evaluates every "[function]" parameter and the mesh vectors
// with muparser (Function.h:8-49, macros.h:35-41, 51-60): variables t (time),
// d (packing density), x, y, z; the constant pi (Function.h:15); muparser's
// operators and functions.  This is an independent parser of that language:
//   precedence (low to high)  ?:   ||   &&   == != < > <= >=   + -   * /
//                             unary -/+   ^ (right associative)
//   functions  sin cos tan asin acos atan sinh cosh tanh asinh acosh atanh
//              exp ln log log2 log10 sqrt sign rint abs min max sum avg
//   constants  pi _pi _e
//   a top-level comma separates the components of a vector ("1,2,3").
// Comparisons and logic give 1 or 0.  ln and log are the natural logarithm
// (muparser's log is natural).
#ifndef SHL_EXPR_H_
#define SHL_EXPR_H_

#include <cctype>
#include <cmath>
#include <cstdlib>
#include <cstring>
#include <map>
#include <memory>
#include <stdexcept>
#include <string>
#include <vector>

namespace shl {
namespace expr {

// A flat program for a stack machine (compiled from an Expression), so that
// the device can evaluate a parameter at its own time (one thread).
enum OpCode : int32_t {
  OP_CONST, OP_VAR, OP_NEG, OP_ADD, OP_SUB, OP_MUL, OP_DIV, OP_POW, OP_LT, OP_GT, OP_LE, OP_GE, OP_EQ, OP_NE,
  OP_AND, OP_OR, OP_FUN1, OP_MIN, OP_MAX, OP_SUM, OP_AVG, OP_JZ, OP_JMP
};
enum Fun1 : int32_t {
  F_SIN, F_COS, F_TAN, F_ASIN, F_ACOS, F_ATAN, F_SINH, F_COSH, F_TANH, F_ASINH, F_ACOSH, F_ATANH, F_EXP, F_LOG,
  F_LOG2, F_LOG10, F_SQRT, F_SIGN, F_RINT, F_ABS
};
struct Op {
  int32_t code;
  int32_t arg;   // variable index (t, d, x, y, z), function id, argument count, or jump target
  double value;  // constant
};
constexpr int kMaxProgram = 256;
constexpr int kMaxStack = 32;

struct Node {
  enum Kind { NUM, VAR, NEG, BIN, FUN, IF } kind = NUM;
  double value = 0;
  std::string name;  // variable or function name, or the operator
  std::vector<std::unique_ptr<Node>> args;
};

class Expression {
 public:
  Expression() = default;
  explicit Expression(const std::string& text) : text_(text) {
    pos_ = 0;
    do {
      roots_.push_back(parse_ternary());
      skip();
    } while (accept(","));
    skip();
    if (pos_ != text_.size()) fail("unexpected '" + text_.substr(pos_, 1) + "'");
  }

  // number of comma-separated components
  size_t size() const { return roots_.size(); }
  // names of the variables the expression reads
  std::vector<std::string> variables() const {
    std::vector<std::string> out;
    for (const auto& r : roots_) collect(r.get(), out);
    return out;
  }
  bool uses(const std::string& var) const {
    for (const auto& v : variables())
      if (v == var) return true;
    return false;
  }
  bool is_constant() const { return variables().empty(); }
  double eval(const std::map<std::string, double>& vars, size_t component = 0) const {
    return eval(roots_.at(component).get(), vars);
  }
  const std::string& text() const { return text_; }

  // program of one component; throws if it exceeds kMaxProgram ops or kMaxStack depth
  std::vector<Op> compile(size_t component = 0) const {
    std::vector<Op> prog;
    int depth = 0, max_depth = 0;
    emit(roots_.at(component).get(), prog, depth, max_depth);
    if ((int)prog.size() > kMaxProgram || max_depth > kMaxStack)
      throw std::runtime_error("expression \"" + text_ + "\" is too long for the device");
    return prog;
  }

 private:
  std::string text_;
  size_t pos_ = 0;
  std::vector<std::unique_ptr<Node>> roots_;

  [[noreturn]] void fail(const std::string& why) const {
    throw std::runtime_error("expression \"" + text_ + "\": " + why);
  }
  void skip() {
    while (pos_ < text_.size() && std::isspace((unsigned char)text_[pos_])) ++pos_;
  }
  bool accept(const char* tok) {
    skip();
    const size_t n = std::char_traits<char>::length(tok);
    if (text_.compare(pos_, n, tok) == 0) {
      pos_ += n;
      return true;
    }
    return false;
  }
  static std::unique_ptr<Node> bin(const char* op, std::unique_ptr<Node> a, std::unique_ptr<Node> b) {
    auto n = std::make_unique<Node>();
    n->kind = Node::BIN;
    n->name = op;
    n->args.push_back(std::move(a));
    n->args.push_back(std::move(b));
    return n;
  }
  std::unique_ptr<Node> parse_ternary() {
    auto c = parse_or();
    if (accept("?")) {
      auto a = parse_ternary();
      if (!accept(":")) fail("missing ':'");
      auto b = parse_ternary();
      auto n = std::make_unique<Node>();
      n->kind = Node::IF;
      n->args.push_back(std::move(c));
      n->args.push_back(std::move(a));
      n->args.push_back(std::move(b));
      return n;
    }
    return c;
  }
  std::unique_ptr<Node> parse_or() {
    auto a = parse_and();
    while (accept("||")) a = bin("||", std::move(a), parse_and());
    return a;
  }
  std::unique_ptr<Node> parse_and() {
    auto a = parse_cmp();
    while (accept("&&")) a = bin("&&", std::move(a), parse_cmp());
    return a;
  }
  std::unique_ptr<Node> parse_cmp() {
    auto a = parse_add();
    for (;;) {
      const char* ops[] = {"==", "!=", "<=", ">=", "<", ">"};
      bool hit = false;
      for (const char* op : ops)
        if (accept(op)) {
          a = bin(op, std::move(a), parse_add());
          hit = true;
          break;
        }
      if (!hit) return a;
    }
  }
  std::unique_ptr<Node> parse_add() {
    auto a = parse_mul();
    for (;;) {
      if (accept("+"))
        a = bin("+", std::move(a), parse_mul());
      else if (accept("-"))
        a = bin("-", std::move(a), parse_mul());
      else
        return a;
    }
  }
  std::unique_ptr<Node> parse_mul() {
    auto a = parse_unary();
    for (;;) {
      if (accept("*"))
        a = bin("*", std::move(a), parse_unary());
      else if (accept("/"))
        a = bin("/", std::move(a), parse_unary());
      else
        return a;
    }
  }
  std::unique_ptr<Node> parse_unary() {
    if (accept("-")) {
      auto n = std::make_unique<Node>();
      n->kind = Node::NEG;
      n->args.push_back(parse_unary());
      return n;
    }
    if (accept("+")) return parse_unary();
    return parse_pow();
  }
  std::unique_ptr<Node> parse_pow() {
    auto a = parse_primary();
    if (accept("^")) return bin("^", std::move(a), parse_unary());
    return a;
  }
  std::unique_ptr<Node> parse_primary() {
    skip();
    if (pos_ >= text_.size()) fail("unexpected end");
    const char c = text_[pos_];
    if (accept("(")) {
      auto e = parse_ternary();
      if (!accept(")")) fail("missing ')'");
      return e;
    }
    if (std::isdigit((unsigned char)c) || c == '.') {
      const char* s = text_.c_str() + pos_;
      char* end = nullptr;
      const double v = std::strtod(s, &end);
      if (end == s) fail("bad number");
      pos_ += (size_t)(end - s);
      auto n = std::make_unique<Node>();
      n->value = v;
      return n;
    }
    if (std::isalpha((unsigned char)c) || c == '_') {
      size_t b = pos_;
      while (pos_ < text_.size() && (std::isalnum((unsigned char)text_[pos_]) || text_[pos_] == '_')) ++pos_;
      const std::string id = text_.substr(b, pos_ - b);
      if (accept("(")) {
        auto n = std::make_unique<Node>();
        n->kind = Node::FUN;
        n->name = id;
        if (!accept(")")) {
          do n->args.push_back(parse_ternary());
          while (accept(","));
          if (!accept(")")) fail("missing ')' after the arguments of " + id);
        }
        check_function(*n);
        return n;
      }
      auto n = std::make_unique<Node>();
      if (id == "pi" || id == "_pi") {
        n->value = 3.141592653589793238462643383279502884;
      } else if (id == "_e") {
        n->value = 2.718281828459045235360287471352662498;
      } else if (id == "t" || id == "d" || id == "x" || id == "y" || id == "z") {
        n->kind = Node::VAR;
        n->name = id;
      } else {
        fail("unknown name '" + id + "'");
      }
      return n;
    }
    fail(std::string("unexpected '") + c + "'");
  }
  void check_function(const Node& n) const {
    static const char* unary[] = {"sin",  "cos",  "tan",   "asin", "acos", "atan", "sinh", "cosh", "tanh",
                                  "asinh", "acosh", "atanh", "exp", "ln",   "log",  "log2", "log10", "sqrt",
                                  "sign", "rint", "abs"};
    for (const char* f : unary)
      if (n.name == f) {
        if (n.args.size() != 1) fail(n.name + " takes one argument");
        return;
      }
    if (n.name == "min" || n.name == "max" || n.name == "sum" || n.name == "avg") {
      if (n.args.empty()) fail(n.name + " needs arguments");
      return;
    }
    fail("unknown function '" + n.name + "'");
  }
  static void push(std::vector<Op>& p, int32_t code, int32_t arg, double value, int& depth, int& max_depth,
                   int pops, int pushes) {
    p.push_back(Op{code, arg, value});
    depth += pushes - pops;
    if (depth > max_depth) max_depth = depth;
  }
  void emit(const Node* n, std::vector<Op>& p, int& depth, int& max_depth) const {
    switch (n->kind) {
      case Node::NUM: push(p, OP_CONST, 0, n->value, depth, max_depth, 0, 1); return;
      case Node::VAR: {
        const char* names = "tdxyz";
        const int idx = (int)(std::strchr(names, n->name[0]) - names);
        push(p, OP_VAR, idx, 0, depth, max_depth, 0, 1);
        return;
      }
      case Node::NEG:
        emit(n->args[0].get(), p, depth, max_depth);
        push(p, OP_NEG, 0, 0, depth, max_depth, 1, 1);
        return;
      case Node::IF: {
        emit(n->args[0].get(), p, depth, max_depth);
        const size_t jz = p.size();
        push(p, OP_JZ, 0, 0, depth, max_depth, 1, 0);
        emit(n->args[1].get(), p, depth, max_depth);
        const size_t jmp = p.size();
        push(p, OP_JMP, 0, 0, depth, max_depth, 0, 0);
        depth -= 1;  // only one branch's value stays on the stack
        p[jz].arg = (int32_t)p.size();
        emit(n->args[2].get(), p, depth, max_depth);
        p[jmp].arg = (int32_t)p.size();
        return;
      }
      case Node::BIN: {
        emit(n->args[0].get(), p, depth, max_depth);
        emit(n->args[1].get(), p, depth, max_depth);
        static const char* ops[] = {"+", "-", "*", "/", "^", "<", ">", "<=", ">=", "==", "!=", "&&", "||"};
        static const int32_t codes[] = {OP_ADD, OP_SUB, OP_MUL, OP_DIV, OP_POW, OP_LT, OP_GT,
                                        OP_LE,  OP_GE,  OP_EQ,  OP_NE,  OP_AND, OP_OR};
        for (int k = 0; k < 13; ++k)
          if (n->name == ops[k]) {
            push(p, codes[k], 0, 0, depth, max_depth, 2, 1);
            return;
          }
        return;
      }
      case Node::FUN: {
        for (const auto& a : n->args) emit(a.get(), p, depth, max_depth);
        static const char* f1[] = {"sin",   "cos",   "tan", "asin", "acos", "atan", "sinh",  "cosh", "tanh", "asinh",
                                   "acosh", "atanh", "exp", "log",  "log2", "log10", "sqrt", "sign", "rint", "abs"};
        for (int k = 0; k < 20; ++k)
          if (n->name == f1[k]) {
            push(p, OP_FUN1, k, 0, depth, max_depth, 1, 1);
            return;
          }
        if (n->name == "ln") {
          push(p, OP_FUN1, F_LOG, 0, depth, max_depth, 1, 1);
          return;
        }
        const int cnt = (int)n->args.size();
        const int32_t code = n->name == "min" ? OP_MIN : n->name == "max" ? OP_MAX : n->name == "sum" ? OP_SUM : OP_AVG;
        push(p, code, cnt, 0, depth, max_depth, cnt, 1);
        return;
      }
    }
  }
  static void collect(const Node* n, std::vector<std::string>& out) {
    if (n->kind == Node::VAR) {
      for (const auto& v : out)
        if (v == n->name) return;
      out.push_back(n->name);
    }
    for (const auto& a : n->args) collect(a.get(), out);
  }
  double eval(const Node* n, const std::map<std::string, double>& vars) const {
    switch (n->kind) {
      case Node::NUM: return n->value;
      case Node::VAR: {
        auto it = vars.find(n->name);
        return it == vars.end() ? 0.0 : it->second;
      }
      case Node::NEG: return -eval(n->args[0].get(), vars);
      case Node::IF:
        return eval(n->args[0].get(), vars) != 0 ? eval(n->args[1].get(), vars) : eval(n->args[2].get(), vars);
      case Node::BIN: {
        const double a = eval(n->args[0].get(), vars), b = eval(n->args[1].get(), vars);
        const std::string& o = n->name;
        if (o == "+") return a + b;
        if (o == "-") return a - b;
        if (o == "*") return a * b;
        if (o == "/") return a / b;
        if (o == "^") return std::pow(a, b);
        if (o == "<") return a < b;
        if (o == ">") return a > b;
        if (o == "<=") return a <= b;
        if (o == ">=") return a >= b;
        if (o == "==") return a == b;
        if (o == "!=") return a != b;
        if (o == "&&") return a != 0 && b != 0;
        if (o == "||") return a != 0 || b != 0;
        return 0;
      }
      case Node::FUN: {
        std::vector<double> x;
        for (const auto& a : n->args) x.push_back(eval(a.get(), vars));
        const std::string& f = n->name;
        if (f == "sin") return std::sin(x[0]);
        if (f == "cos") return std::cos(x[0]);
        if (f == "tan") return std::tan(x[0]);
        if (f == "asin") return std::asin(x[0]);
        if (f == "acos") return std::acos(x[0]);
        if (f == "atan") return std::atan(x[0]);
        if (f == "sinh") return std::sinh(x[0]);
        if (f == "cosh") return std::cosh(x[0]);
        if (f == "tanh") return std::tanh(x[0]);
        if (f == "asinh") return std::asinh(x[0]);
        if (f == "acosh") return std::acosh(x[0]);
        if (f == "atanh") return std::atanh(x[0]);
        if (f == "exp") return std::exp(x[0]);
        if (f == "ln" || f == "log") return std::log(x[0]);
        if (f == "log2") return std::log2(x[0]);
        if (f == "log10") return std::log10(x[0]);
        if (f == "sqrt") return std::sqrt(x[0]);
        if (f == "sign") return (x[0] > 0) - (x[0] < 0);
        if (f == "rint") return std::rint(x[0]);
        if (f == "abs") return std::fabs(x[0]);
        double r = x[0];
        if (f == "min")
          for (double v : x) r = v < r ? v : r;
        if (f == "max")
          for (double v : x) r = v > r ? v : r;
        if (f == "sum" || f == "avg") {
          r = 0;
          for (double v : x) r += v;
          if (f == "avg") r /= (double)x.size();
        }
        return r;
      }
    }
    return 0;
  }
};

}  // namespace expr
}  // namespace shl

#endif
