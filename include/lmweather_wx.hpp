/* The wx.* operator surface of lmweather (cpp/main.cpp:62-494) over the GPU engine: the 81 methods of the Wx,
 * Sphere and Plane types, with the reference's names, parameter and return kinds, argument checks, builder
 * initialisers, text writers and error texts, registered against the C ABI through the C++ classes of
 * lmweather_gb300.hpp. Header-only; link with liblmw_gb300.so.
 *
 * register_host<VM>(registry, host) is written against a small VM interface so the same registrations serve two
 * registries:
 *   - the scripting VM lmweather embeds (dslvm::Registry, dslvm::Value, dslvm::Args, dslvm::Error), through
 *     a traits struct { using Registry = dslvm::Registry; using Value = dslvm::Value; using Args = dslvm::Args;
 *     using Error = dslvm::Error; }: the host program's register_host call is the only line that changes;
 *   - MiniVM below, a registry of this library that calls methods by name (the lmw_wx_* C ABI and its tests use it)
 *     and writes the registry's schema as JSON in the layout of schema/lmweather.dsl.json.
 * The VM's Value needs: kind (VOID, INT, FLOAT, STR, BOOL, OBJ), fields i, f, s, b, obj, type, and the factories
 * none, integer, real, string, boolean, object; its Error is constructible from a message string.
 *
 * Expression strings (Sphere.fields/orography/tracer, Plane.fields) are compiled by Expr below, which accepts the
 * grammar of cpp/expr.hpp with its limits and error texts and evaluates it as a postfix program. */
#ifndef LMWEATHER_WX_HPP
#define LMWEATHER_WX_HPP

#include <cctype>
#include <cerrno>
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <fstream>
#include <functional>
#include <iostream>
#include <map>
#include <memory>
#include <stdexcept>
#include <string>
#include <utility>
#include <vector>

#include "lmweather_gb300.hpp"

namespace lmweather_gb300 {
namespace wx {

// the reference release whose operator surface this layer reproduces (CMakeLists.txt:2)
constexpr const char *kInterfaceVersion = "0.1.4";

// ------------------------------------------------------------------------------------------------ expressions
// Arithmetic over named variables and constants (cpp/expr.hpp:15-158). Grammar, lowest precedence first:
//   sum   := product (('+' | '-') product)*
//   product := signed (('*' | '/') signed)*
//   signed  := '-' signed | '+' signed | power
//   power := atom (('^' | '**') signed)?          right-associative; the exponent may carry a sign
//   atom  := '(' sum ')' | number | name '(' [sum (',' sum)*] ')' | name
// Names resolve to a variable, then a parameter, then pi and e. Functions: sin cos tan asin acos atan sinh cosh tanh
// exp log ln log10 sqrt abs floor ceil sign (one argument), atan2 pow min max mod (two). The sum and signed rules
// each count one nesting level (at most 200) and every atom one term (at most 2000), so deep or long strings are
// errors, not stack overflows. Errors are std::runtime_error
//   expression "<text, cut to 117 characters and '...' past 120>": <what> at column <1-based position>.
// The compiled form is a postfix program run on a value stack: evaluation does not recurse.
class Expr {
 public:
  Expr(const std::string &text, const std::vector<std::string> &vars, const std::map<std::string, double> &params = {})
      : text_(text), vars_(vars), params_(params) {
    sum();
    skip();
    if (at_ != text_.size()) fail(std::string("unexpected '") + text_[at_] + "'");
  }

  double eval(const double *x) const {
    double small[32];
    std::vector<double> big;
    double *st = small;
    if (depth_max_ > 32) {
      big.resize(depth_max_);
      st = big.data();
    }
    int sp = 0;
    for (const Ins &c : code_) {
      switch (c.op) {
        case K: st[sp++] = c.k; break;
        case X: st[sp++] = x[c.slot]; break;
        case NEG: st[sp - 1] = -st[sp - 1]; break;
        case F1: st[sp - 1] = c.f1(st[sp - 1]); break;
        default: {
          const double b = st[--sp], a = st[sp - 1];
          double r;
          switch (c.op) {
            case ADD: r = a + b; break;
            case SUB: r = a - b; break;
            case MUL: r = a * b; break;
            case DIV: r = a / b; break;
            case POW: r = std::pow(a, b); break;
            default: r = c.f2(a, b); break;
          }
          st[sp - 1] = r;
        }
      }
    }
    return st[0];
  }

 private:
  enum Op : unsigned char { K, X, NEG, ADD, SUB, MUL, DIV, POW, F1, F2 };
  struct Ins {
    Op op;
    int slot;
    double k;
    double (*f1)(double);
    double (*f2)(double, double);
  };
  static constexpr int kMaxNesting = 200;
  static constexpr int kMaxTerms = 2000;

  std::string text_;
  std::vector<std::string> vars_;
  std::map<std::string, double> params_;
  std::vector<Ins> code_;
  size_t at_ = 0;
  int nesting_ = 0, terms_ = 0, depth_ = 0, depth_max_ = 1;

  struct Level {
    Expr &e;
    explicit Level(Expr &x) : e(x) {
      if (++e.nesting_ > kMaxNesting) e.fail("expression is nested too deeply");
    }
    ~Level() { --e.nesting_; }
  };

  [[noreturn]] void fail(const std::string &what) const {
    const std::string shown = text_.size() <= 120 ? text_ : text_.substr(0, 117) + "...";
    throw std::runtime_error("expression \"" + shown + "\": " + what + " at column " + std::to_string(at_ + 1));
  }
  void skip() {
    while (at_ < text_.size() && std::isspace(static_cast<unsigned char>(text_[at_]))) at_++;
  }
  bool take(char c) {
    skip();
    if (at_ < text_.size() && text_[at_] == c) {
      at_++;
      return true;
    }
    return false;
  }
  bool take_starstar() {
    skip();
    if (at_ + 1 < text_.size() && text_[at_] == '*' && text_[at_ + 1] == '*') {
      at_ += 2;
      return true;
    }
    return false;
  }
  // stack effect of each instruction, tracked so eval() can size its stack
  void emit(Op op, int slot = 0, double k = 0, double (*f1)(double) = nullptr, double (*f2)(double, double) = nullptr) {
    code_.push_back(Ins{op, slot, k, f1, f2});
    if (op == K || op == X) {
      if (++depth_ > depth_max_) depth_max_ = depth_;
    } else if (op != NEG && op != F1) {
      depth_--;
    }
  }

  void sum() {
    Level lv(*this);
    product();
    for (;;) {
      if (take('+')) {
        product();
        emit(ADD);
      } else if (take('-')) {
        product();
        emit(SUB);
      } else {
        return;
      }
    }
  }
  void product() {
    signed_term();
    for (;;) {
      if (take('*')) {
        signed_term();
        emit(MUL);
      } else if (take('/')) {
        signed_term();
        emit(DIV);
      } else {
        return;
      }
    }
  }
  void signed_term() {
    Level lv(*this);
    if (take('-')) {
      signed_term();
      emit(NEG);
    } else if (take('+')) {
      signed_term();
    } else {
      power();
    }
  }
  void power() {
    atom();
    if (take('^') || take_starstar()) {
      signed_term();
      emit(POW);
    }
  }
  void atom() {
    skip();
    if (at_ >= text_.size()) fail("unexpected end");
    const char c = text_[at_];
    if (++terms_ > kMaxTerms) fail("expression has too many terms");
    if (c == '(') {
      at_++;
      sum();
      if (!take(')')) fail("expected ')'");
      return;
    }
    if (std::isdigit(static_cast<unsigned char>(c)) || c == '.') {
      const char *start = text_.c_str() + at_;
      char *end = nullptr;
      errno = 0;
      const double v = std::strtod(start, &end);
      if (end == start || errno == ERANGE) fail("number is malformed or out of range");
      at_ += static_cast<size_t>(end - start);
      emit(K, 0, v);
      return;
    }
    if (std::isalpha(static_cast<unsigned char>(c)) || c == '_') {
      const size_t s = at_;
      while (at_ < text_.size() && (std::isalnum(static_cast<unsigned char>(text_[at_])) || text_[at_] == '_')) at_++;
      const std::string name = text_.substr(s, at_ - s);
      skip();
      if (at_ < text_.size() && text_[at_] == '(') {
        at_++;
        int nargs = 0;
        if (!take(')')) {
          do {
            sum();
            nargs++;
          } while (take(','));
          if (!take(')')) fail("expected ')'");
        }
        function(name, nargs);
        return;
      }
      for (size_t i = 0; i < vars_.size(); i++)
        if (vars_[i] == name) {
          emit(X, static_cast<int>(i));
          return;
        }
      const auto p = params_.find(name);
      if (p != params_.end()) {
        emit(K, 0, p->second);
        return;
      }
      if (name == "pi") {
        emit(K, 0, 3.14159265358979323846);
        return;
      }
      if (name == "e") {
        emit(K, 0, 2.71828182845904523536);
        return;
      }
      fail("unknown name '" + name + "'");
    }
    fail(std::string("unexpected '") + c + "'");
  }
  // the arguments are compiled (and their errors raised) before the name and the count are checked
  void function(const std::string &f, int nargs) {
    using U = double (*)(double);
    using B = double (*)(double, double);
    static const std::map<std::string, U> one = {
        {"sin", [](double x) { return std::sin(x); }},     {"cos", [](double x) { return std::cos(x); }},
        {"tan", [](double x) { return std::tan(x); }},     {"asin", [](double x) { return std::asin(x); }},
        {"acos", [](double x) { return std::acos(x); }},   {"atan", [](double x) { return std::atan(x); }},
        {"sinh", [](double x) { return std::sinh(x); }},   {"cosh", [](double x) { return std::cosh(x); }},
        {"tanh", [](double x) { return std::tanh(x); }},   {"exp", [](double x) { return std::exp(x); }},
        {"log", [](double x) { return std::log(x); }},     {"ln", [](double x) { return std::log(x); }},
        {"log10", [](double x) { return std::log10(x); }}, {"sqrt", [](double x) { return std::sqrt(x); }},
        {"abs", [](double x) { return std::fabs(x); }},    {"floor", [](double x) { return std::floor(x); }},
        {"ceil", [](double x) { return std::ceil(x); }},
        {"sign", [](double x) { return static_cast<double>((x > 0) - (x < 0)); }}};
    static const std::map<std::string, B> two = {{"atan2", [](double y, double x) { return std::atan2(y, x); }},
                                                 {"pow", [](double a, double b) { return std::pow(a, b); }},
                                                 {"min", [](double a, double b) { return a < b ? a : b; }},
                                                 {"max", [](double a, double b) { return a > b ? a : b; }},
                                                 {"mod", [](double a, double b) { return std::fmod(a, b); }}};
    const auto u = one.find(f);
    if (u != one.end()) {
      if (nargs != 1) fail(f + " takes 1 argument");
      emit(F1, 0, 0, u->second);
      return;
    }
    const auto b = two.find(f);
    if (b != two.end()) {
      if (nargs != 2) fail(f + " takes 2 arguments");
      emit(F2, 0, 0, nullptr, b->second);
      return;
    }
    fail("unknown function '" + f + "'");
  }
};

// ------------------------------------------------------------------------------------------------ MiniVM
// A registry that calls methods by name: the interface register_host needs, plus call() and the schema.
struct MiniVM {
  struct Value {
    enum Kind { VOID, INT, FLOAT, STR, BOOL, OBJ } kind = VOID;
    int64_t i = 0;
    double f = 0.0;
    std::string s;
    bool b = false;
    void *obj = nullptr;
    std::string type;  // the type name of obj
    static Value none() { return Value(); }
    static Value integer(int64_t v) {
      Value x;
      x.kind = INT;
      x.i = v;
      return x;
    }
    static Value real(double v) {
      Value x;
      x.kind = FLOAT;
      x.f = v;
      return x;
    }
    static Value string(std::string v) {
      Value x;
      x.kind = STR;
      x.s = std::move(v);
      return x;
    }
    static Value boolean(bool v) {
      Value x;
      x.kind = BOOL;
      x.b = v;
      return x;
    }
    static Value object(const std::string &t, void *p) {
      Value x;
      x.kind = OBJ;
      x.obj = p;
      x.type = t;
      return x;
    }
  };
  using Args = std::vector<Value>;
  using Method = std::function<Value(void *, Args &)>;
  struct Error : std::runtime_error {
    explicit Error(const std::string &m) : std::runtime_error(m) {}
  };

  class Registry {
   public:
    struct Entry {
      std::string type, name;
      std::vector<std::string> params;
      std::string returns;
      Method fn;
    };
    Registry &method(const std::string &type, const std::string &name, std::vector<std::string> params, std::string returns, Method fn) {
      for (const Entry &e : entries_)
        if (e.type == type && e.name == name) throw Error("registry: method " + type + "." + name + " is registered twice");
      entries_.push_back(Entry{type, name, std::move(params), std::move(returns), std::move(fn)});
      return *this;
    }
    Registry &context(const std::string &name, const std::string &type) {
      for (const auto &c : context_)
        if (c.first == name) throw Error("registry: context '" + name + "' is declared twice");
      context_.emplace_back(name, type);
      return *this;
    }
    const Entry *find(const std::string &type, const std::string &name) const {
      for (const Entry &e : entries_)
        if (e.type == type && e.name == name) return &e;
      return nullptr;
    }
    const std::vector<Entry> &entries() const { return entries_; }
    // the registry as schema JSON: types in the order their first method was registered, methods in registration
    // order, each a one-element overload list; two-space indentation and a final newline
    std::string schema_json(const std::string &name) const {
      std::vector<std::string> types;
      for (const Entry &e : entries_) {
        bool seen = false;
        for (const auto &t : types) seen = seen || t == e.type;
        if (!seen) types.push_back(e.type);
      }
      auto q = [](const std::string &s) { return "\"" + s + "\""; };
      std::string o = "{\n  \"dsl.schema\": 2,\n  \"name\": " + q(name) + ",\n  \"types\": {";
      for (size_t ti = 0; ti < types.size(); ti++) {
        o += (ti ? ",\n" : "\n") + std::string(4, ' ') + q(types[ti]) + ": {\n      \"methods\": {";
        bool first = true;
        for (const Entry &e : entries_) {
          if (e.type != types[ti]) continue;
          o += (first ? "\n" : ",\n") + std::string(8, ' ') + q(e.name) + ": [\n" + std::string(10, ' ') + "{\n" +
               std::string(12, ' ') + "\"params\": ";
          if (e.params.empty()) {
            o += "[]";
          } else {
            o += "[";
            for (size_t k = 0; k < e.params.size(); k++) o += (k ? ",\n" : "\n") + std::string(14, ' ') + q(e.params[k]);
            o += "\n" + std::string(12, ' ') + "]";
          }
          o += ",\n" + std::string(12, ' ') + "\"returns\": " + q(e.returns) + "\n" + std::string(10, ' ') + "}\n" +
               std::string(8, ' ') + "]";
          first = false;
        }
        o += "\n      }\n    }";
      }
      o += types.empty() ? "}" : "\n  }";
      o += ",\n  \"functions\": {},\n  \"context\": {";
      for (size_t c = 0; c < context_.size(); c++) o += (c ? ",\n" : "\n") + std::string(4, ' ') + q(context_[c].first) + ": " + q(context_[c].second);
      o += context_.empty() ? "}" : "\n  }";
      return o + "\n}\n";
    }

   private:
    std::vector<Entry> entries_;
    std::vector<std::pair<std::string, std::string>> context_;
  };
};

// ------------------------------------------------------------------------------------------------ host objects
constexpr double kPi = 3.14159265358979323846;
constexpr double kDeg = kPi / 180.0;

struct SphereObj {
  std::unique_ptr<Sphere> model;
};
struct PlaneObj {
  PlaneParams params;
  std::unique_ptr<Plane> model;
  bool started = false;  // fields were set: depth() would reset them
};

// The objects scripts create (cpp/main.cpp:35-54): owned here and freed with the host, at most 100,000 of each type.
struct Host {
  static constexpr size_t kMaxObjects = 100000;
  std::vector<std::unique_ptr<SphereObj>> spheres;
  std::vector<std::unique_ptr<PlaneObj>> planes;
  // where Wx.print writes (standard output unless the embedding program redirects it)
  std::function<void(const std::string &)> print = [](const std::string &s) { std::cout << s << '\n' << std::flush; };

  bool owns(const std::string &type, const void *p) const {
    if (type == "Sphere") {
      for (const auto &o : spheres)
        if (o.get() == p) return true;
    } else if (type == "Plane") {
      for (const auto &o : planes)
        if (o.get() == p) return true;
    }
    return false;
  }
};

namespace detail {
inline std::string num17(double x) {
  char b[48];
  std::snprintf(b, sizeof b, "%.17g", x);
  return b;
}
inline void write_file(const std::string &path, const std::string &text, const char *who) {
  std::ofstream f(path, std::ios::binary);
  if (!f) throw std::runtime_error(std::string(who) + ": cannot write " + path);
  f << text;
  f.flush();
  if (!f) throw std::runtime_error(std::string(who) + ": cannot write " + path);
}
}  // namespace detail

// Registers the Wx, Sphere and Plane methods (cpp/main.cpp:96-494) in registration order.
template <class VM> void register_host(typename VM::Registry &r, Host &host) {
  using Value = typename VM::Value;
  using Args = typename VM::Args;
  using Error = typename VM::Error;
  using Fn = std::function<Value(void *, Args &)>;

  // The checked registration of cpp/main.cpp:62-80: argument kinds are checked against the declared ones, any
  // std::exception from the engine becomes the VM's error with the same text, and a float result must be finite.
  auto method = [&r](const char *type, const char *name, std::vector<std::string> ps, std::string ret, Fn fn) {
    const std::string who = std::string(type) + "." + name;
    const bool real = ret == "float";
    r.method(type, name, ps, ret, [who, ps, fn, real](void *self, Args &a) -> Value {
      if (a.size() != ps.size()) throw Error(who + " takes " + std::to_string(ps.size()) + " argument(s), got " + std::to_string(a.size()));
      for (size_t i = 0; i < ps.size(); ++i) {
        const Value &p = a[i];
        bool ok;
        if (ps[i] == "float") ok = p.kind == Value::FLOAT;
        else if (ps[i] == "int") ok = p.kind == Value::INT;
        else if (ps[i] == "string") ok = p.kind == Value::STR;
        else if (ps[i] == "bool") ok = p.kind == Value::BOOL;
        else ok = p.kind == Value::OBJ && p.obj && p.type == ps[i];
        if (!ok) throw Error(who + " argument " + std::to_string(i + 1) + " must be " + ps[i]);
      }
      Value out;
      try {
        out = fn(self, a);
      } catch (const Error &) {
        throw;
      } catch (const std::exception &e) {
        throw Error(e.what());
      }
      if (real && out.kind == Value::FLOAT && !std::isfinite(out.f)) throw Error(who + ": the result is not finite");
      return out;
    });
  };
  auto need = [](bool ok, const std::string &msg) {
    if (!ok) throw Error(msg);
  };
  auto finite = [need](double x, const char *what) {
    need(std::isfinite(x), std::string(what) + " must be a finite number");
    return x;
  };
  // an int argument passed on as a C int: values a cast would wrap are refused
  auto narrow = [need](int64_t v, const char *who) {
    need(v >= -1000000000 && v <= 1000000000, std::string(who) + ": integer argument out of range");
    return static_cast<int>(v);
  };
  auto positive = [need](double x, const std::string &msg) {
    need(std::isfinite(x) && x > 0, msg);
    return x;
  };
  auto latitude = [need](double deg, const char *who) {
    need(std::fabs(deg) <= 90.0, std::string(who) + ": latitude must be within +-90 degrees");
    return deg * kDeg;
  };
  auto self_sphere = [](void *p) -> Sphere & { return *static_cast<SphereObj *>(p)->model; };
  auto self_plane = [](void *p) -> PlaneObj & { return *static_cast<PlaneObj *>(p); };
  auto same_sphere = [](void *p) { return Value::object("Sphere", p); };
  auto same_plane = [](void *p) { return Value::object("Plane", p); };
  // a grid of one expression per point, in the reference's row order (latitude rows south to north)
  auto on_grid = [](const Sphere &m, const Expr &e, std::vector<double> &out) {
    out.resize(static_cast<size_t>(m.nlat()) * m.nlon());
    for (int j = 0; j < m.nlat(); j++)
      for (int k = 0; k < m.nlon(); k++) {
        const double x[2] = {m.lon(k), m.lat(j)};
        out[static_cast<size_t>(j) * m.nlon() + k] = e.eval(x);
      }
  };
  auto sphere_constants = [](const Sphere &m) {
    const SphereParams &sp = m.params();
    return std::map<std::string, double>{{"a", sp.radius}, {"omega", sp.omega}, {"g", sp.gravity}};
  };

  r.context("wx", "Wx");
  // ---------------------------------------------------------------- Wx (cpp/main.cpp:98-145)
  auto make_sphere = [&host, need](int64_t n, const SphereParams &sp) {
    need(n >= 4 && n <= 170, "Wx.sphere: truncation must be between 4 and 170");
    need(std::isfinite(sp.radius) && std::isfinite(sp.gravity) && std::isfinite(sp.omega) && sp.radius > 0 && sp.gravity > 0 && sp.omega >= 0,
         "Wx.planet: radius and gravity must be positive and omega not negative");
    need(host.spheres.size() < Host::kMaxObjects, "Sphere object limit exceeded");
    auto o = std::make_unique<SphereObj>();
    o->model = std::make_unique<Sphere>(static_cast<int>(n), sp);
    host.spheres.push_back(std::move(o));
    return Value::object("Sphere", host.spheres.back().get());
  };
  method("Wx", "sphere", {"int"}, "Sphere", [make_sphere](void *, Args &a) { return make_sphere(a[0].i, SphereParams{}); });
  method("Wx", "planet", {"int", "float", "float", "float"}, "Sphere", [make_sphere](void *, Args &a) {
    SphereParams sp;
    sp.radius = a[1].f;
    sp.omega = a[2].f;
    sp.gravity = a[3].f;
    return make_sphere(a[0].i, sp);
  });
  method("Wx", "plane", {"int", "int", "float", "float"}, "Plane", [&host, need](void *, Args &a) {
    need(a[0].i >= 4 && a[1].i >= 4 && a[0].i <= 4000 && a[1].i <= 4000 && a[0].i * a[1].i <= 8000000,
         "Wx.plane: need 4..4000 cells each way and at most 8 million cells");
    need(std::isfinite(a[2].f) && std::isfinite(a[3].f) && a[2].f > 0 && a[3].f > 0, "Wx.plane: domain sizes must be positive (m)");
    need(host.planes.size() < Host::kMaxObjects, "Plane object limit exceeded");
    auto o = std::make_unique<PlaneObj>();
    o->params.nx = static_cast<int>(a[0].i);
    o->params.ny = static_cast<int>(a[1].i);
    o->params.lx = a[2].f;
    o->params.ly = a[3].f;
    o->model = std::make_unique<Plane>(o->params);
    host.planes.push_back(std::move(o));
    return Value::object("Plane", host.planes.back().get());
  });
  method("Wx", "assert_close", {"float", "float", "float"}, "void", [](void *, Args &a) {
    const double x = a[0].f, y = a[1].f, tol = a[2].f;
    if (!std::isfinite(x) || !std::isfinite(y) || !std::isfinite(tol) || tol < 0 || std::fabs(x - y) > tol)
      throw Error("assert_close failed: " + detail::num17(x) + " vs " + detail::num17(y) + " (tolerance " + detail::num17(tol) + ")");
    return Value::none();
  });
  method("Wx", "assert_true", {"bool"}, "void", [](void *, Args &a) {
    if (!a[0].b) throw Error("assert_true failed");
    return Value::none();
  });
  method("Wx", "print", {"string"}, "void", [&host](void *, Args &a) {
    host.print(a[0].s);
    return Value::none();
  });
  method("Wx", "save_text", {"string", "string"}, "void", [](void *, Args &a) {
    detail::write_file(a[0].s, a[1].s, "Wx.save_text");
    return Value::none();
  });
  method("Wx", "version", {}, "string", [](void *, Args &) { return Value::string(std::string("lmweather ") + kInterfaceVersion); });

  // ---------------------------------------------------------------- Sphere (cpp/main.cpp:147-357)
  auto S = self_sphere;
  method("Sphere", "tilt", {"float"}, "Sphere", [S, finite, same_sphere](void *p, Args &a) {
    S(p).set_axis_tilt(finite(a[0].f, "tilt angle"));
    return same_sphere(p);
  });
  method("Sphere", "diffusion", {"float"}, "Sphere", [S, need, same_sphere](void *p, Args &a) {
    need(std::isfinite(a[0].f) && a[0].f >= 0, "Sphere.diffusion: coefficient must be finite and not negative");
    S(p).set_diffusion(a[0].f);
    return same_sphere(p);
  });
  method("Sphere", "fields", {"string", "string", "string"}, "Sphere", [S, need, on_grid, sphere_constants, same_sphere](void *p, Args &a) {
    Sphere &m = S(p);
    const auto par = sphere_constants(m);
    const Expr eh(a[0].s, {"lon", "lat"}, par), eu(a[1].s, {"lon", "lat"}, par), ev(a[2].s, {"lon", "lat"}, par);
    std::vector<double> hh, uu, vv;
    on_grid(m, eh, hh);
    on_grid(m, eu, uu);
    on_grid(m, ev, vv);
    for (size_t i = 0; i < hh.size(); i++) need(std::isfinite(hh[i] + uu[i] + vv[i]), "Sphere.fields: an expression is not finite on the grid");
    m.set_state_grid(hh, uu, vv);
    return same_sphere(p);
  });
  // Williamson et al. (1992) test case 2: steady zonal flow about an axis tilted by alpha
  method("Sphere", "williamson2", {"float"}, "Sphere", [S, finite, same_sphere](void *p, Args &a) {
    Sphere &m = S(p);
    const SphereParams &sp = m.params();
    const double al = finite(a[0].f, "angle"), u0 = 2 * kPi * sp.radius / (12 * 86400.0), h0 = 2.94e4 / sp.gravity;
    m.set_axis_tilt(al);
    const size_t n = static_cast<size_t>(m.nlat()) * m.nlon();
    std::vector<double> hh(n), uu(n), vv(n);
    for (int j = 0; j < m.nlat(); j++)
      for (int k = 0; k < m.nlon(); k++) {
        const double lat = m.lat(j), lon = m.lon(k);
        const size_t i = static_cast<size_t>(j) * m.nlon() + k;
        uu[i] = u0 * (std::cos(lat) * std::cos(al) + std::sin(lat) * std::cos(lon) * std::sin(al));
        vv[i] = -u0 * std::sin(lon) * std::sin(al);
        const double t = -std::cos(lon) * std::cos(lat) * std::sin(al) + std::sin(lat) * std::cos(al);
        hh[i] = h0 - (sp.radius * sp.omega * u0 + 0.5 * u0 * u0) * t * t / sp.gravity;
      }
    m.set_state_grid(hh, uu, vv);
    return same_sphere(p);
  });
  // test case 6: the Rossby-Haurwitz wave of zonal wavenumber 4
  method("Sphere", "williamson6", {}, "Sphere", [S, same_sphere](void *p, Args &) {
    Sphere &m = S(p);
    const SphereParams &sp = m.params();
    const double w = 7.848e-6, K = 7.848e-6, R = 4, h0 = 8000, ra = sp.radius, Om = sp.omega;
    m.set_axis_tilt(0);
    const size_t n = static_cast<size_t>(m.nlat()) * m.nlon();
    std::vector<double> hh(n), uu(n), vv(n);
    for (int j = 0; j < m.nlat(); j++)
      for (int k = 0; k < m.nlon(); k++) {
        const double ph = m.lat(j), la = m.lon(k), c = std::cos(ph), sn = std::sin(ph);
        const size_t i = static_cast<size_t>(j) * m.nlon() + k;
        uu[i] = ra * w * c + ra * K * std::pow(c, R - 1) * (R * sn * sn - c * c) * std::cos(R * la);
        vv[i] = -ra * K * R * std::pow(c, R - 1) * sn * std::sin(R * la);
        const double A = w / 2 * (2 * Om + w) * c * c + K * K / 4 * std::pow(c, 2 * R) * ((R + 1) * c * c + (2 * R * R - R - 2) - 2 * R * R / (c * c));
        const double B = 2 * (Om + w) * K / ((R + 1) * (R + 2)) * std::pow(c, R) * ((R * R + 2 * R + 2) - (R + 1) * (R + 1) * c * c);
        const double C = K * K / 4 * std::pow(c, 2 * R) * ((R + 1) * c * c - (R + 2));
        hh[i] = h0 + ra * ra / sp.gravity * (A + B * std::cos(R * la) + C * std::cos(2 * R * la));
      }
    m.set_state_grid(hh, uu, vv);
    return same_sphere(p);
  });
  method("Sphere", "orography", {"string"}, "Sphere", [S, need, on_grid, sphere_constants, same_sphere](void *p, Args &a) {
    Sphere &m = S(p);
    const Expr es(a[0].s, {"lon", "lat"}, sphere_constants(m));
    std::vector<double> hs;
    on_grid(m, es, hs);
    for (double x : hs) need(std::isfinite(x), "Sphere.orography: the expression is not finite on the grid");
    m.set_orography_grid(hs);
    return same_sphere(p);
  });
  // test case 5: zonal flow (20 m/s, 5960 m) over a conical mountain of 2000 m, radius pi/9, at 270 E 30 N; the
  // free surface is that of test case 2 and the fluid thickness is the free surface minus the mountain
  method("Sphere", "williamson5", {}, "Sphere", [S, same_sphere](void *p, Args &) {
    Sphere &m = S(p);
    const SphereParams &sp = m.params();
    const double u0 = 20.0, h0 = 5960.0, hs0 = 2000.0, R = kPi / 9, lonc = 1.5 * kPi, latc = kPi / 6;
    m.set_axis_tilt(0);
    const size_t n = static_cast<size_t>(m.nlat()) * m.nlon();
    std::vector<double> hh(n), uu(n), vv(n, 0.0), hs(n);
    for (int j = 0; j < m.nlat(); j++)
      for (int k = 0; k < m.nlon(); k++) {
        const double lat = m.lat(j), lon = m.lon(k);
        const size_t i = static_cast<size_t>(j) * m.nlon() + k;
        const double rr = std::sqrt(std::min(R * R, (lon - lonc) * (lon - lonc) + (lat - latc) * (lat - latc)));
        hs[i] = hs0 * (1 - rr / R);
        uu[i] = u0 * std::cos(lat);
        hh[i] = h0 - (sp.radius * sp.omega * u0 + 0.5 * u0 * u0) * std::sin(lat) * std::sin(lat) / sp.gravity - hs[i];
      }
    m.set_orography_grid(hs);
    m.set_state_grid(hh, uu, vv);
    return same_sphere(p);
  });
  method("Sphere", "tracer", {"string"}, "Sphere", [S, need, on_grid, sphere_constants, same_sphere](void *p, Args &a) {
    Sphere &m = S(p);
    const Expr eq(a[0].s, {"lon", "lat"}, sphere_constants(m));
    std::vector<double> qq;
    on_grid(m, eq, qq);
    for (double x : qq) need(std::isfinite(x), "Sphere.tracer: the expression is not finite on the grid");
    m.set_tracer_grid(qq);
    return same_sphere(p);
  });
  method("Sphere", "advect_only", {}, "Sphere", [S, same_sphere](void *p, Args &) {
    S(p).set_advect_only(true);
    return same_sphere(p);
  });
  // test case 1: a cosine bell (1000 m, radius a/3, at 270 E on the equator) carried once around the globe in 12 days
  // by solid-body rotation about an axis tilted by alpha; the winds are prescribed (advect-only)
  method("Sphere", "williamson1", {"float"}, "Sphere", [S, finite, same_sphere](void *p, Args &a) {
    Sphere &m = S(p);
    const SphereParams &sp = m.params();
    const double al = finite(a[0].f, "angle"), u0 = 2 * kPi * sp.radius / (12 * 86400.0), R = sp.radius / 3, lonc = 1.5 * kPi, latc = 0;
    m.set_axis_tilt(al);
    const size_t n = static_cast<size_t>(m.nlat()) * m.nlon();
    std::vector<double> hh(n, 1000.0), uu(n), vv(n), qq(n);
    for (int j = 0; j < m.nlat(); j++)
      for (int k = 0; k < m.nlon(); k++) {
        const double lat = m.lat(j), lon = m.lon(k);
        const size_t i = static_cast<size_t>(j) * m.nlon() + k;
        uu[i] = u0 * (std::cos(lat) * std::cos(al) + std::sin(lat) * std::cos(lon) * std::sin(al));
        vv[i] = -u0 * std::sin(lon) * std::sin(al);
        const double c = std::sin(latc) * std::sin(lat) + std::cos(latc) * std::cos(lat) * std::cos(lon - lonc);
        const double rr = sp.radius * std::acos(std::max(-1.0, std::min(1.0, c)));
        qq[i] = rr < R ? 500.0 * (1 + std::cos(kPi * rr / R)) : 0.0;
      }
    m.set_state_grid(hh, uu, vv);
    m.set_tracer_grid(qq);
    m.set_advect_only(true);
    return same_sphere(p);
  });
  // the latitude is checked before the longitude
  auto at_point = [latitude, finite](Args &a, const char *who, const char *lon_what) {
    const double lat = latitude(a[0].f, who);
    return std::make_pair(lat, finite(a[1].f, lon_what) * kDeg);
  };
  method("Sphere", "tracer_at", {"float", "float"}, "float", [S, at_point](void *p, Args &a) {
    const auto ll = at_point(a, "Sphere.tracer_at", "Sphere.tracer_at: longitude");
    return Value::real(S(p).tracer_at(ll.first, ll.second));
  });
  method("Sphere", "tracer_mean", {}, "float", [S](void *p, Args &) { return Value::real(S(p).tracer_mean()); });
  method("Sphere", "tracer_mass", {}, "float", [S](void *p, Args &) { return Value::real(S(p).tracer_mass()); });
  method("Sphere", "tracer_min", {}, "float", [S](void *p, Args &) { return Value::real(S(p).tracer_min()); });
  method("Sphere", "tracer_max", {}, "float", [S](void *p, Args &) { return Value::real(S(p).tracer_max()); });
  method("Sphere", "tracer_error_l2", {}, "float", [S](void *p, Args &) { return Value::real(S(p).tracer_error_l2()); });
  method("Sphere", "tracer_error_linf", {}, "float", [S](void *p, Args &) { return Value::real(S(p).tracer_error_linf()); });
  method("Sphere", "mode", {"int", "int", "float", "float"}, "Sphere", [S, positive, narrow, finite, same_sphere](void *p, Args &a) {
    positive(a[3].f, "Sphere.mode: mean depth must be positive");
    const int n = narrow(a[0].i, "Sphere.mode"), m = narrow(a[1].i, "Sphere.mode");
    S(p).add_mode(n, m, finite(a[2].f, "amplitude"), a[3].f);
    return same_sphere(p);
  });
  method("Sphere", "perturb", {"float", "int", "int"}, "Sphere", [S, need, finite, narrow, same_sphere](void *p, Args &a) {
    need(a[1].i >= 0, "Sphere.perturb: seed must not be negative");
    const double amp = finite(a[0].f, "amplitude");
    S(p).perturb(amp, static_cast<uint64_t>(a[1].i), narrow(a[2].i, "Sphere.perturb"));
    return same_sphere(p);
  });
  method("Sphere", "mark_reference", {}, "Sphere", [S, same_sphere](void *p, Args &) {
    S(p).mark_reference();
    return same_sphere(p);
  });
  method("Sphere", "run", {"float"}, "Sphere", [S, finite, same_sphere](void *p, Args &a) {
    S(p).run(finite(a[0].f, "seconds"), 0);
    return same_sphere(p);
  });
  method("Sphere", "run_dt", {"float", "float"}, "Sphere", [S, positive, finite, same_sphere](void *p, Args &a) {
    positive(a[1].f, "Sphere.run_dt: dt must be positive");
    S(p).run(finite(a[0].f, "seconds"), a[1].f);
    return same_sphere(p);
  });
  method("Sphere", "stable_dt", {}, "float", [S](void *p, Args &) { return Value::real(S(p).stable_dt()); });
  method("Sphere", "time", {}, "float", [S](void *p, Args &) { return Value::real(S(p).time()); });
  method("Sphere", "truncation", {}, "int", [S](void *p, Args &) { return Value::integer(S(p).truncation()); });
  method("Sphere", "nlat", {}, "int", [S](void *p, Args &) { return Value::integer(S(p).nlat()); });
  method("Sphere", "nlon", {}, "int", [S](void *p, Args &) { return Value::integer(S(p).nlon()); });
  method("Sphere", "mean_height", {}, "float", [S](void *p, Args &) { return Value::real(S(p).mean_height()); });
  method("Sphere", "energy", {}, "float", [S](void *p, Args &) { return Value::real(S(p).energy()); });
  method("Sphere", "kinetic_energy", {}, "float", [S](void *p, Args &) { return Value::real(S(p).kinetic_energy()); });
  method("Sphere", "potential_energy", {}, "float", [S](void *p, Args &) { return Value::real(S(p).potential_energy()); });
  // the text files are written by the engine from the device state (lmw_sphere_save_*)
  method("Sphere", "save_spectrum", {"string"}, "void", [S](void *p, Args &a) {
    check(lmw_sphere_save_spectrum(S(p).handle(), 0, a[0].s.c_str()));
    return Value::none();
  });
  method("Sphere", "enstrophy", {}, "float", [S](void *p, Args &) { return Value::real(S(p).potential_enstrophy()); });
  method("Sphere", "max_wind", {}, "float", [S](void *p, Args &) { return Value::real(S(p).max_wind()); });
  method("Sphere", "error_l2", {}, "float", [S](void *p, Args &) { return Value::real(S(p).height_error_l2()); });
  method("Sphere", "error_linf", {}, "float", [S](void *p, Args &) { return Value::real(S(p).height_error_linf()); });
  method("Sphere", "height_at", {"float", "float"}, "float", [S, at_point](void *p, Args &a) {
    const auto ll = at_point(a, "Sphere.height_at", "Sphere.height_at: longitude");
    return Value::real(S(p).height_at(ll.first, ll.second));
  });
  method("Sphere", "u_at", {"float", "float"}, "float", [S, need, finite](void *p, Args &a) {
    need(std::fabs(a[0].f) < 90.0, "Sphere.u_at: latitude must be inside (-90, 90) degrees");
    return Value::real(S(p).wind_at(a[0].f * kDeg, finite(a[1].f, "Sphere.u_at: longitude") * kDeg, true));
  });
  method("Sphere", "v_at", {"float", "float"}, "float", [S, need, finite](void *p, Args &a) {
    need(std::fabs(a[0].f) < 90.0, "Sphere.v_at: latitude must be inside (-90, 90) degrees");
    return Value::real(S(p).wind_at(a[0].f * kDeg, finite(a[1].f, "Sphere.v_at: longitude") * kDeg, false));
  });
  method("Sphere", "vorticity_at", {"float", "float"}, "float", [S, at_point](void *p, Args &a) {
    const auto ll = at_point(a, "Sphere.vorticity_at", "Sphere.vorticity_at: longitude");
    return Value::real(S(p).vorticity_at(ll.first, ll.second));
  });
  method("Sphere", "mode_coefficient", {"int", "int", "string"}, "float", [S, need, narrow](void *p, Args &a) {
    need(a[2].s == "re" || a[2].s == "im", "Sphere.mode_coefficient: part must be re or im");
    const int n = narrow(a[0].i, "Sphere.mode_coefficient"), m = narrow(a[1].i, "Sphere.mode_coefficient");
    return Value::real(S(p).mode_coefficient(n, m, a[2].s == "im"));
  });
  method("Sphere", "wave_crest", {"int", "float"}, "float", [S, narrow, latitude](void *p, Args &a) {
    const int m = narrow(a[0].i, "Sphere.wave_crest");
    return Value::real(S(p).wave_crest(m, latitude(a[1].f, "Sphere.wave_crest")) / kDeg);
  });
  method("Sphere", "save_csv", {"string"}, "void", [S](void *p, Args &a) {
    check(lmw_sphere_save_csv(S(p).handle(), 0, a[0].s.c_str()));
    return Value::none();
  });
  method("Sphere", "save_zonal_mean", {"string"}, "void", [S](void *p, Args &a) {
    check(lmw_sphere_save_zonal_mean(S(p).handle(), 0, a[0].s.c_str()));
    return Value::none();
  });

  // ---------------------------------------------------------------- Plane (cpp/main.cpp:387-494)
  auto P = self_plane;
  // the parameters live in the object; every setter pushes them to the engine
  auto sync = [](PlaneObj &o) {
    o.model->params() = o.params;
    o.model->apply_params();
  };
  method("Plane", "gravity", {"float"}, "Plane", [P, positive, sync, same_plane](void *p, Args &a) {
    positive(a[0].f, "Plane.gravity: must be positive");
    P(p).params.gravity = a[0].f;
    sync(P(p));
    return same_plane(p);
  });
  method("Plane", "depth", {"float"}, "Plane", [P, positive, need, sync, same_plane](void *p, Args &a) {
    positive(a[0].f, "Plane.depth: must be positive (m)");
    need(!P(p).started, "Plane.depth: set the depth before fields() or perturb()");
    P(p).params.depth = a[0].f;
    sync(P(p));
    P(p).model->reset();
    return same_plane(p);
  });
  method("Plane", "coriolis", {"float", "float"}, "Plane", [P, finite, sync, same_plane](void *p, Args &a) {
    P(p).params.f0 = finite(a[0].f, "f0");
    P(p).params.beta = finite(a[1].f, "beta");
    sync(P(p));
    return same_plane(p);
  });
  method("Plane", "linear", {}, "Plane", [P, sync, same_plane](void *p, Args &) {
    P(p).params.linear = true;
    sync(P(p));
    return same_plane(p);
  });
  method("Plane", "nonlinear", {}, "Plane", [P, sync, same_plane](void *p, Args &) {
    P(p).params.linear = false;
    sync(P(p));
    return same_plane(p);
  });
  method("Plane", "viscosity", {"float"}, "Plane", [P, need, sync, same_plane](void *p, Args &a) {
    need(std::isfinite(a[0].f) && a[0].f >= 0, "Plane.viscosity: must be finite and not negative");
    P(p).params.viscosity = a[0].f;
    sync(P(p));
    return same_plane(p);
  });
  method("Plane", "drag", {"float"}, "Plane", [P, need, sync, same_plane](void *p, Args &a) {
    need(std::isfinite(a[0].f) && a[0].f >= 0, "Plane.drag: must be finite and not negative");
    P(p).params.drag = a[0].f;
    sync(P(p));
    return same_plane(p);
  });
  // h = H + expression at cell centres, u at west faces, v at the interior south faces (the walls keep v = 0)
  method("Plane", "fields", {"string", "string", "string"}, "Plane", [P, need, same_plane](void *p, Args &a) {
    PlaneObj &o = P(p);
    Plane &m = *o.model;
    const PlaneParams &q = o.params;
    const std::map<std::string, double> par{{"lx", q.lx}, {"ly", q.ly}, {"H", q.depth}, {"g", q.gravity}, {"f0", q.f0}, {"beta", q.beta}};
    const Expr eh(a[0].s, {"x", "y"}, par), eu(a[1].s, {"x", "y"}, par), ev(a[2].s, {"x", "y"}, par);
    const int nx = q.nx, ny = q.ny;
    std::vector<double> hh(static_cast<size_t>(nx) * ny), uu(hh.size()), vv(static_cast<size_t>(nx) * (ny + 1), 0.0);
    for (int j = 0; j < ny; j++)
      for (int i = 0; i < nx; i++) {
        const double xc[2] = {m.x_center(i), m.y_center(j)}, xu[2] = {i * m.dx(), m.y_center(j)};
        hh[static_cast<size_t>(j) * nx + i] = q.depth + eh.eval(xc);
        uu[static_cast<size_t>(j) * nx + i] = eu.eval(xu);
      }
    for (int j = 1; j < ny; j++)
      for (int i = 0; i < nx; i++) {
        const double xv[2] = {m.x_center(i), j * m.dy()};
        vv[static_cast<size_t>(j) * nx + i] = ev.eval(xv);
      }
    for (double x : hh) need(std::isfinite(x), "Plane.fields: the height expression is not finite");
    for (double x : uu) need(std::isfinite(x), "Plane.fields: the u expression is not finite");
    for (double x : vv) need(std::isfinite(x), "Plane.fields: the v expression is not finite");
    m.set_h_from_grid(hh);
    m.set_u_from_grid(uu);
    m.set_v_from_grid(vv);
    o.started = true;
    return same_plane(p);
  });
  method("Plane", "perturb", {"float", "int"}, "Plane", [P, need, finite, same_plane](void *p, Args &a) {
    need(a[1].i >= 0, "Plane.perturb: seed must not be negative");
    P(p).model->perturb(finite(a[0].f, "amplitude"), static_cast<uint64_t>(a[1].i));
    P(p).started = true;
    return same_plane(p);
  });
  method("Plane", "run", {"float"}, "Plane", [P, finite, same_plane](void *p, Args &a) {
    P(p).model->run(finite(a[0].f, "seconds"), 0);
    P(p).started = true;
    return same_plane(p);
  });
  method("Plane", "run_dt", {"float", "float"}, "Plane", [P, positive, finite, same_plane](void *p, Args &a) {
    positive(a[1].f, "Plane.run_dt: dt must be positive");
    P(p).model->run(finite(a[0].f, "seconds"), a[1].f);
    P(p).started = true;
    return same_plane(p);
  });
  method("Plane", "stable_dt", {}, "float", [P](void *p, Args &) { return Value::real(P(p).model->stable_dt()); });
  method("Plane", "time", {}, "float", [P](void *p, Args &) { return Value::real(P(p).model->time()); });
  method("Plane", "wave_speed", {}, "float", [P](void *p, Args &) { return Value::real(std::sqrt(P(p).params.gravity * P(p).params.depth)); });
  method("Plane", "rossby_radius", {}, "float", [P, need](void *p, Args &) {
    need(P(p).params.f0 != 0, "Plane.rossby_radius: f0 is zero");
    return Value::real(std::sqrt(P(p).params.gravity * P(p).params.depth) / std::fabs(P(p).params.f0));
  });
  method("Plane", "mean_depth", {}, "float", [P](void *p, Args &) { return Value::real(P(p).model->mean_depth()); });
  method("Plane", "energy", {}, "float", [P](void *p, Args &) { return Value::real(P(p).model->energy()); });
  method("Plane", "max_speed", {}, "float", [P](void *p, Args &) { return Value::real(P(p).model->max_speed()); });
  method("Plane", "pv_anomaly_rms", {}, "float", [P](void *p, Args &) { return Value::real(P(p).model->potential_vorticity_anomaly_rms()); });
  auto inside = [P, need](void *p, double x, double y, const char *who) {
    need(x >= 0 && x <= P(p).params.lx && y >= 0 && y <= P(p).params.ly, std::string(who) + ": point outside the domain");
  };
  method("Plane", "h_at", {"float", "float"}, "float", [P, inside](void *p, Args &a) {
    inside(p, a[0].f, a[1].f, "Plane.h_at");
    return Value::real(P(p).model->h_at(a[0].f, a[1].f));
  });
  method("Plane", "u_at", {"float", "float"}, "float", [P, inside](void *p, Args &a) {
    inside(p, a[0].f, a[1].f, "Plane.u_at");
    return Value::real(P(p).model->u_at(a[0].f, a[1].f));
  });
  method("Plane", "v_at", {"float", "float"}, "float", [P, inside](void *p, Args &a) {
    inside(p, a[0].f, a[1].f, "Plane.v_at");
    return Value::real(P(p).model->v_at(a[0].f, a[1].f));
  });
  method("Plane", "zonal_amplitude", {"int", "int"}, "float", [P, narrow](void *p, Args &a) {
    const int m = narrow(a[0].i, "Plane.zonal_amplitude"), j = narrow(a[1].i, "Plane.zonal_amplitude");
    return Value::real(P(p).model->zonal_amplitude(m, j));
  });
  method("Plane", "zonal_crest", {"int", "int"}, "float", [P, narrow](void *p, Args &a) {
    const int m = narrow(a[0].i, "Plane.zonal_crest"), j = narrow(a[1].i, "Plane.zonal_crest");
    return Value::real(P(p).model->zonal_crest(m, j));
  });
  method("Plane", "harmonic_energy", {"int"}, "float", [P, narrow](void *p, Args &a) {
    return Value::real(P(p).model->harmonic_energy(narrow(a[0].i, "Plane.harmonic_energy")));
  });
  method("Plane", "v_zonal_crest", {"int", "int"}, "float", [P, narrow](void *p, Args &a) {
    const int m = narrow(a[0].i, "Plane.v_zonal_crest"), j = narrow(a[1].i, "Plane.v_zonal_crest");
    return Value::real(P(p).model->v_zonal_crest(m, j));
  });
  method("Plane", "save_csv", {"string"}, "void", [P](void *p, Args &a) {
    check(lmw_plane_save_csv(P(p).model->handle(), a[0].s.c_str()));
    return Value::none();
  });
  // the row and column are checked here as 64-bit values, before they are passed on as C ints
  method("Plane", "save_row", {"int", "string"}, "void", [P, need](void *p, Args &a) {
    need(a[0].i >= 0 && a[0].i < P(p).params.ny, "Plane.save_row: row outside the grid");
    check(lmw_plane_save_row(P(p).model->handle(), static_cast<int>(a[0].i), a[1].s.c_str()));
    return Value::none();
  });
  method("Plane", "save_column", {"int", "string"}, "void", [P, need](void *p, Args &a) {
    need(a[0].i >= 0 && a[0].i < P(p).params.nx, "Plane.save_column: column outside the grid");
    check(lmw_plane_save_column(P(p).model->handle(), static_cast<int>(a[0].i), a[1].s.c_str()));
    return Value::none();
  });
}

}  // namespace wx
}  // namespace lmweather_gb300

#endif
