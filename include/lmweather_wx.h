/* lmweather-gb300: C ABI of the wx.* operator surface (lmweather cpp/main.cpp:62-494) over the GPU engine.
 *
 * A host (lmw_wx) owns the Sphere and Plane objects that its calls create and the registry of the 81 methods of
 * the Wx, Sphere and Plane types (include/lmweather_wx.hpp). lmw_wx_call invokes one method by type and name with
 * the reference's argument kinds, checks and error texts: the reference turns every failure inside a method into a
 * run error of its scripting VM (cpp/main.cpp:56-60), and here every such failure returns LMW_RUNTIME_ERROR with
 * that text in lmw_last_error(). Status codes as in lmweather_gb300.h. */
#ifndef LMWEATHER_WX_H
#define LMWEATHER_WX_H

#include <stddef.h>
#include <stdint.h>

#include "lmweather_gb300.h"

#ifdef __cplusplus
extern "C" {
#endif

/* value kinds of the scripting VM (cpp/dslvm.hpp Value::Kind, without the dry-run kind) */
enum { LMW_WX_VOID = 0, LMW_WX_INT = 1, LMW_WX_FLOAT = 2, LMW_WX_STR = 3, LMW_WX_BOOL = 4, LMW_WX_OBJ = 5 };

typedef struct lmw_wx lmw_wx;
typedef struct lmw_wx_value {
  int kind;
  int64_t i;     /* LMW_WX_INT; LMW_WX_BOOL as 0 or 1 */
  double f;      /* LMW_WX_FLOAT */
  const char *s; /* LMW_WX_STR: NUL-terminated text; LMW_WX_OBJ: the object's type name ("Sphere" or "Plane") */
  void *obj;     /* LMW_WX_OBJ: an object this host returned */
} lmw_wx_value;

/* the host of cpp/main.cpp:35-54 with every method registered (cpp/main.cpp:96-494) */
int lmw_wx_create(lmw_wx **out);
/* frees the host and every object it created */
int lmw_wx_destroy(lmw_wx *h);
/* type.method(args) on self (an object of that type that this host returned; ignored for type "Wx", the context
 * object). ret receives the result; a string result stays valid until the host's next call, an object result until
 * the host is destroyed. LMW_INVALID_ARGUMENT for an unknown method, a foreign object or a wrong argument count
 * (the scripting VM refuses those when it loads a program); LMW_RUNTIME_ERROR with the reference's message for
 * every failure inside the method, including an argument of the wrong kind ("<Type.method> argument <k> must be
 * <kind>") and a non-finite float result ("<Type.method>: the result is not finite"). */
int lmw_wx_call(lmw_wx *h, const char *type, void *self, const char *method, const lmw_wx_value *args, int nargs, lmw_wx_value *ret);
/* the registry as schema JSON, byte for byte the layout of lmweather's schema/lmweather.dsl.json (scripts/gen-schema.py):
 * *len receives its length in bytes; when buf is not NULL it must hold len + 1 bytes and receives the text and a NUL */
int lmw_wx_schema(lmw_wx *h, char *buf, size_t cap, size_t *len);
/* the engine handle behind a Sphere or Plane object of this host, for the entry points beyond the wx methods (state
 * I/O, precision, timing); owned by the object */
int lmw_wx_sphere_handle(lmw_wx *h, void *obj, lmw_sphere **out);
int lmw_wx_plane_handle(lmw_wx *h, void *obj, lmw_plane **out);
/* The expression compiler of the builders (cpp/expr.hpp): compiles text over the n variables `names` and evaluates
 * it at `values`. LMW_RUNTIME_ERROR with the reference's message ("expression \"...\": <what> at column <k>") when
 * the text does not compile. */
int lmw_expr_eval(const char *text, const char *const *names, const double *values, int n, double *out);

#ifdef __cplusplus
}
#endif

#endif
