// C ABI of the wx.* operator surface (include/lmweather_wx.h): a host with the registrations of
// include/lmweather_wx.hpp on this library's own registry, methods called by type and name.
#include <cstring>
#include <string>
#include <vector>

#include "lmw_internal.h"
#include "lmweather_wx.h"
#include "lmweather_wx.hpp"

namespace wx = lmweather_gb300::wx;
using VM = wx::MiniVM;

struct lmw_wx {
  wx::Host host;
  VM::Registry reg;
  std::string text;  // the last string result
};

namespace {
void need(bool ok, const std::string &msg) {
  if (!ok) throw lmw::InvalidArgument(msg);
}

VM::Value to_value(const lmw_wx &h, const lmw_wx_value &a, int k) {
  const std::string at = "argument " + std::to_string(k + 1);
  switch (a.kind) {
    case LMW_WX_INT: return VM::Value::integer(a.i);
    case LMW_WX_FLOAT: return VM::Value::real(a.f);
    case LMW_WX_BOOL: return VM::Value::boolean(a.i != 0);
    case LMW_WX_STR:
      need(a.s != nullptr, at + ": string is null");
      return VM::Value::string(a.s);
    case LMW_WX_OBJ:
      need(a.s != nullptr && h.host.owns(a.s, a.obj), at + ": not an object of this host");
      return VM::Value::object(a.s, a.obj);
    case LMW_WX_VOID: return VM::Value::none();
    default: throw lmw::InvalidArgument(at + ": unknown value kind " + std::to_string(a.kind));
  }
}
}  // namespace

extern "C" {

int lmw_wx_create(lmw_wx **out) {
  return lmw::run_guarded([&] {
    need(out != nullptr, "output handle pointer is null");
    *out = nullptr;
    auto *h = new lmw_wx();
    try {
      wx::register_host<VM>(h->reg, h->host);
    } catch (...) {
      delete h;
      throw;
    }
    *out = h;
  });
}

int lmw_wx_destroy(lmw_wx *h) {
  return lmw::run_guarded([&] { delete h; });
}

int lmw_wx_call(lmw_wx *h, const char *type, void *self, const char *method, const lmw_wx_value *args, int nargs, lmw_wx_value *ret) {
  return lmw::run_guarded([&] {
    need(h != nullptr && type != nullptr && method != nullptr && ret != nullptr, "null host, type, method or result pointer");
    need(nargs >= 0 && (nargs == 0 || args != nullptr), "argument array is null");
    const VM::Registry::Entry *e = h->reg.find(type, method);
    need(e != nullptr, std::string("unknown method ") + type + "." + method);
    need(static_cast<size_t>(nargs) == e->params.size(),
         e->type + "." + e->name + " takes " + std::to_string(e->params.size()) + " argument(s), got " + std::to_string(nargs));
    if (e->type != "Wx") need(h->host.owns(e->type, self), e->type + "." + e->name + ": the receiver is not a " + e->type + " of this host");
    VM::Args a;
    a.reserve(nargs);
    for (int k = 0; k < nargs; k++) a.push_back(to_value(*h, args[k], k));
    VM::Value r = e->fn(e->type == "Wx" ? static_cast<void *>(h) : self, a);
    *ret = lmw_wx_value{LMW_WX_VOID, 0, 0.0, nullptr, nullptr};
    switch (r.kind) {
      case VM::Value::VOID: break;
      case VM::Value::INT:
        ret->kind = LMW_WX_INT;
        ret->i = r.i;
        break;
      case VM::Value::FLOAT:
        ret->kind = LMW_WX_FLOAT;
        ret->f = r.f;
        break;
      case VM::Value::BOOL:
        ret->kind = LMW_WX_BOOL;
        ret->i = r.b ? 1 : 0;
        break;
      case VM::Value::STR:
        h->text = r.s;
        ret->kind = LMW_WX_STR;
        ret->s = h->text.c_str();
        break;
      case VM::Value::OBJ:
        ret->kind = LMW_WX_OBJ;
        ret->obj = r.obj;
        ret->s = e->returns.c_str();  // the registry's type name, stable while the host lives
        break;
    }
  });
}

int lmw_wx_schema(lmw_wx *h, char *buf, size_t cap, size_t *len) {
  return lmw::run_guarded([&] {
    need(h != nullptr && len != nullptr, "null host or length pointer");
    const std::string s = h->reg.schema_json("lmweather");
    *len = s.size();
    if (buf != nullptr) {
      need(cap > s.size(), "schema buffer too small");
      std::memcpy(buf, s.c_str(), s.size() + 1);
    }
  });
}

int lmw_wx_sphere_handle(lmw_wx *h, void *obj, lmw_sphere **out) {
  return lmw::run_guarded([&] {
    need(h != nullptr && out != nullptr, "null host or output pointer");
    need(h->host.owns("Sphere", obj), "not a Sphere of this host");
    *out = static_cast<wx::SphereObj *>(obj)->model->handle();
  });
}

int lmw_wx_plane_handle(lmw_wx *h, void *obj, lmw_plane **out) {
  return lmw::run_guarded([&] {
    need(h != nullptr && out != nullptr, "null host or output pointer");
    need(h->host.owns("Plane", obj), "not a Plane of this host");
    *out = static_cast<wx::PlaneObj *>(obj)->model->handle();
  });
}

int lmw_expr_eval(const char *text, const char *const *names, const double *values, int n, double *out) {
  return lmw::run_guarded([&] {
    need(text != nullptr && out != nullptr && n >= 0 && (n == 0 || (names != nullptr && values != nullptr)), "null expression, names, values or output");
    std::vector<std::string> vars;
    for (int k = 0; k < n; k++) {
      need(names[k] != nullptr, "variable name is null");
      vars.push_back(names[k]);
    }
    const wx::Expr e(text, vars);
    *out = e.eval(values);
  });
}

}  // extern "C"
