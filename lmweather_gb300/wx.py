"""The wx.* operator surface (lmweather cpp/main.cpp:62-494) from Python, over the C ABI of include/lmweather_wx.h.

    wx = Wx()
    s = wx.sphere(21).williamson2(0.05)
    s.run_dt(432000.0, 1800.0)
    wx.assert_true(s.error_l2() < 1e-6)

reads like the reference's scripts: every method of the Wx, Sphere and Plane types is called by name with the
script's argument kinds (Python int -> int, float -> float, bool -> bool, str -> string, an object -> that
object). A failure inside a method raises WxError with the reference's message (the scripting VM's run error);
an unknown method or a wrong argument count raises ValueError.
"""
from __future__ import annotations

import ctypes as C

from . import _check, load_library

VOID, INT, FLOAT, STR, BOOL, OBJ = 0, 1, 2, 3, 4, 5


class WxError(RuntimeError):
    """A run error of a wx method (status LMW_RUNTIME_ERROR), with the reference's message."""


class _Value(C.Structure):
    _fields_ = [("kind", C.c_int), ("i", C.c_int64), ("f", C.c_double), ("s", C.c_char_p), ("obj", C.c_void_p)]


_SIGS = {
    "lmw_wx_create": (C.c_int, [C.POINTER(C.c_void_p)]),
    "lmw_wx_destroy": (C.c_int, [C.c_void_p]),
    "lmw_wx_call": (C.c_int, [C.c_void_p, C.c_char_p, C.c_void_p, C.c_char_p, C.POINTER(_Value), C.c_int, C.POINTER(_Value)]),
    "lmw_wx_schema": (C.c_int, [C.c_void_p, C.c_char_p, C.c_size_t, C.POINTER(C.c_size_t)]),
    "lmw_wx_sphere_handle": (C.c_int, [C.c_void_p, C.c_void_p, C.POINTER(C.c_void_p)]),
    "lmw_wx_plane_handle": (C.c_int, [C.c_void_p, C.c_void_p, C.POINTER(C.c_void_p)]),
    "lmw_expr_eval": (C.c_int, [C.c_char_p, C.POINTER(C.c_char_p), C.POINTER(C.c_double), C.c_int, C.POINTER(C.c_double)]),
}


def _lib():
    lib = load_library()
    if not getattr(lib, "_wx_bound", False):
        for name, (res, args) in _SIGS.items():
            f = getattr(lib, name)
            f.restype = res
            f.argtypes = args
        lib._wx_bound = True
    return lib


def _status(code: int) -> None:
    if code == 2:
        raise WxError(load_library().lmw_last_error().decode())
    _check(code)


def eval_expression(text: str, **variables: float) -> float:
    """Compile `text` over the given variables with the builders' expression compiler and evaluate it there."""
    lib = _lib()
    names = list(variables)
    arr_n = (C.c_char_p * max(1, len(names)))(*[n.encode() for n in names])
    arr_v = (C.c_double * max(1, len(names)))(*[float(variables[n]) for n in names])
    out = C.c_double()
    _status(lib.lmw_expr_eval(text.encode(), arr_n, arr_v, len(names), C.byref(out)))
    return out.value


class WxObject:
    """A Sphere or Plane the host created; attribute access yields its methods."""

    def __init__(self, host: "Wx", type_: str, ptr: int):
        self._host, self._type, self._ptr = host, type_, ptr

    @property
    def type(self) -> str:
        return self._type

    def engine_handle(self) -> int:
        """The engine handle (lmw_sphere* or lmw_plane*) behind this object, for the C ABI's other entry points."""
        out = C.c_void_p()
        fn = self._host._lib.lmw_wx_sphere_handle if self._type == "Sphere" else self._host._lib.lmw_wx_plane_handle
        _status(fn(self._host._h, self._ptr, C.byref(out)))
        return out.value

    def __getattr__(self, name: str):
        if name.startswith("_"):
            raise AttributeError(name)
        return lambda *args: self._host._call(self._type, self._ptr, name, args)

    def __eq__(self, other) -> bool:
        return isinstance(other, WxObject) and other._ptr == self._ptr

    def __hash__(self) -> int:
        return hash(self._ptr)

    def __repr__(self) -> str:
        return f"<{self._type} 0x{self._ptr:x}>"


class Wx:
    """A wx host: the context object `wx` of the reference's scripts, owner of every object its calls create."""

    def __init__(self):
        self._lib = _lib()
        h = C.c_void_p()
        _status(self._lib.lmw_wx_create(C.byref(h)))
        self._h = h

    def close(self) -> None:
        if getattr(self, "_h", None) and self._h.value:
            self._lib.lmw_wx_destroy(self._h)
            self._h = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def schema(self) -> bytes:
        """The registry as schema JSON (the layout of lmweather's schema/lmweather.dsl.json)."""
        n = C.c_size_t()
        _status(self._lib.lmw_wx_schema(self._h, None, 0, C.byref(n)))
        buf = C.create_string_buffer(n.value + 1)
        _status(self._lib.lmw_wx_schema(self._h, buf, n.value + 1, C.byref(n)))
        return buf.raw[: n.value]

    def __getattr__(self, name: str):
        if name.startswith("_"):
            raise AttributeError(name)
        return lambda *args: self._call("Wx", None, name, args)

    def _call(self, type_: str, ptr, name: str, args):
        vals = (_Value * max(1, len(args)))()
        keep = []
        for k, a in enumerate(args):
            v = vals[k]
            if isinstance(a, bool):
                v.kind, v.i = BOOL, int(a)
            elif isinstance(a, int):
                v.kind, v.i = INT, a
            elif isinstance(a, float):
                v.kind, v.f = FLOAT, a
            elif isinstance(a, str):
                b = a.encode()
                keep.append(b)
                v.kind, v.s = STR, b
            elif isinstance(a, WxObject):
                b = a.type.encode()
                keep.append(b)
                v.kind, v.s, v.obj = OBJ, b, a._ptr
            else:
                raise TypeError(f"{type_}.{name}: argument {k + 1} has no script kind ({type(a).__name__})")
        ret = _Value()
        _status(self._lib.lmw_wx_call(self._h, type_.encode(), ptr, name.encode(), vals, len(args), C.byref(ret)))
        if ret.kind == INT:
            return ret.i
        if ret.kind == FLOAT:
            return ret.f
        if ret.kind == BOOL:
            return bool(ret.i)
        if ret.kind == STR:
            return ret.s.decode()
        if ret.kind == OBJ:
            return WxObject(self, ret.s.decode(), ret.obj)
        return None
