"""A small WGSL interpreter: the subset the reference's compute shaders
(MLS-MPM, SPH) and fullscreen fragment shaders (bilateral and gaussian
filters, shading) use.

TEST INFRASTRUCTURE: make_golden.py, make_golden_sph.py and
make_golden_render.py run the reference's own WGSL source text through this
interpreter to produce golden vectors that pin the C oracles.  It is
independent of the oracles: it parses the shader and evaluates it with
WGSL's static typing and abstract-numeric conversion rules, rounding every
f32 operation separately (numpy float32 scalars).  Compute entry points run
one invocation at a time (dispatch); a fragment entry point is called once
per pixel with its interpolated inputs.

Choices the WGSL specification leaves to the implementation are fixed the
same way the oracles fix them (they cannot be pinned by any source):
  * matrix * vector adds the columns in order: ((c0*v.x + c1*v.y) + c2*v.z) ...;
  * dot(a, b) = (a.x*b.x + a.y*b.y) + a.z*b.z; normalize(v) = v / sqrt(dot(v, v));
    sqrt correctly rounded;
  * pow(x, 5.0) = ((x*x)*(x*x))*x (other exponents through float64 pow) unless
    a generator installs POW_F32; exp is EXP_F32 (float64 exp by default;
    the renderer's generator installs the project's restatement);
  * f32 -> i32 / u32 of NaN is 0; out-of-range conversions saturate (spec);
  * a storage access outside the bound array reads zero and drops writes, and
    is counted once per visit (consecutive accesses to one element);
  * a texture load outside the image reads the nearest edge texel; a cube
    texture is sampled by CUBE_SAMPLE, which a generator installs (filtering
    is the sampling unit's work, not shader arithmetic).
Everything else (operand order, literal conversion, integer wraparound, loop
structure, which fields are read and written) comes from the shader text.
"""
from __future__ import annotations

import math
import re

import numpy as np

F32 = np.float32

# --------------------------------------------------------------------------
# types
# --------------------------------------------------------------------------


class T:
    def __init__(self, kind, elem=None, n=0, fields=None, name=None):
        self.kind = kind      # 'f32','i32','u32','bool','absint','absfloat','vec','mat','array','struct','atomic'
        self.elem = elem
        self.n = n
        self.fields = fields  # list of (name, type) for structs
        self.name = name

    def __repr__(self):
        if self.kind == "vec":
            return f"vec{self.n}<{self.elem}>"
        if self.kind == "mat":
            return f"mat{self.n}x{self.n}<{self.elem}>"
        if self.kind == "array":
            return f"array<{self.elem},{self.n}>"
        if self.kind == "struct":
            return self.name
        return self.kind


TF32, TI32, TU32, TBOOL = T("f32"), T("i32"), T("u32"), T("bool")
TABSI, TABSF = T("absint"), T("absfloat")


def vec(elem, n=3):
    return T("vec", elem, n)


def mat(elem, n=3):
    return T("mat", elem, n)


def is_abstract(t):
    return t.kind in ("absint", "absfloat")


def scalar_of(t):
    if t.kind in ("vec", "mat"):
        return t.elem
    if t.kind == "atomic":
        return t.elem
    return t


def wrap32(x: int) -> int:
    return ((int(x) + 0x80000000) & 0xFFFFFFFF) - 0x80000000


def f2i(x) -> int:
    x = float(x)
    if math.isnan(x):
        return 0
    if x >= 2147483648.0:
        return 2147483647
    if x <= -2147483648.0:
        return -2147483648
    return int(x)  # truncation toward zero


def f2u(x) -> int:
    x = float(x)
    if math.isnan(x) or x <= 0:
        return 0
    if x >= 4294967296.0:
        return 4294967295
    return int(x)


def zero_value(t):
    k = t.kind
    if k == "f32":
        return F32(0)
    if k in ("i32", "u32"):
        return 0
    if k == "bool":
        return False
    if k == "atomic":
        return 0
    if k == "vec":
        return tuple(zero_value(t.elem) for _ in range(t.n))
    if k == "mat":
        return tuple(tuple(F32(0) for _ in range(t.n)) for _ in range(t.n))
    if k == "array":
        return [zero_value(t.elem) for _ in range(t.n)]
    if k == "struct":
        return {f: zero_value(ft) for f, ft in t.fields}
    raise TypeError(t)


def convert(v, src, dst):
    """Converts a value of abstract type src to concrete type dst."""
    if dst.kind in ("vec",):
        return tuple(convert(v, src, dst.elem) for _ in range(dst.n)) if not isinstance(v, tuple) \
            else tuple(convert(x, scalar_of(src), dst.elem) for x in v)
    if dst.kind == "f32":
        return F32(v)
    if dst.kind == "i32":
        return wrap32(int(v))
    if dst.kind == "u32":
        return int(v) & 0xFFFFFFFF
    if dst.kind in ("absfloat",):
        return float(v)
    return v


# --------------------------------------------------------------------------
# lexer
# --------------------------------------------------------------------------

TOKEN_RE = re.compile(r"""
    (?P<ws>\s+|//[^\n]*|/\*.*?\*/)
  | (?P<num>(\d+\.\d*|\.\d+|\d+)([eE][+-]?\d+)?[fiu]?)
  | (?P<id>[A-Za-z_][A-Za-z0-9_]*)
  | (?P<op>->|\+\+|--|\+=|-=|\*=|/=|%=|<=|>=|==|!=|&&|\|\||[-+*/%<>=!&|^(){}\[\],;:.@])
""", re.S | re.X)


def lex(src):
    out = []
    pos = 0
    while pos < len(src):
        m = TOKEN_RE.match(src, pos)
        if not m:
            raise SyntaxError(f"bad character at {pos}: {src[pos:pos + 20]!r}")
        pos = m.end()
        if m.lastgroup == "ws":
            continue
        out.append((m.lastgroup, m.group(m.lastgroup)))
    out.append(("eof", ""))
    return out


# --------------------------------------------------------------------------
# parser -> AST (tuples)
# --------------------------------------------------------------------------

class Parser:
    def __init__(self, src):
        self.toks = lex(src)
        self.i = 0

    def peek(self, k=0):
        return self.toks[self.i + k]

    def next(self):
        t = self.toks[self.i]
        self.i += 1
        return t

    def accept(self, val):
        if self.peek()[1] == val:
            self.i += 1
            return True
        return False

    def expect(self, val):
        t = self.next()
        if t[1] != val:
            raise SyntaxError(f"expected {val!r}, got {t[1]!r} near token {self.i}")
        return t

    def ident(self):
        t = self.next()
        if t[0] != "id":
            raise SyntaxError(f"expected identifier, got {t[1]!r}")
        return t[1]

    # types
    def parse_type(self):
        name = self.ident()
        if name in ("vec2", "vec3", "vec4"):
            self.expect("<")
            e = self.parse_type()
            self.expect(">")
            return ("vec", int(name[3]), e)
        if len(name) == 5 and name[:3] == "vec" and name[3] in "234" and name[4] in "fiu":
            return ("vec", int(name[3]), ({"f": "f32", "i": "i32", "u": "u32"}[name[4]],))
        if name in ("texture_2d", "texture_cube"):
            self.expect("<")
            e = self.parse_type()
            self.expect(">")
            return ("texture" if name == "texture_2d" else "texture_cube", e)
        if name == "sampler":
            return ("sampler",)
        if name == "mat4x4f":
            return ("mat", 4, ("f32",))
        if name == "mat3x3f":
            return ("mat", 3, ("f32",))
        if name == "mat3x3":
            self.expect("<")
            e = self.parse_type()
            self.expect(">")
            return ("mat", 3, e)
        if name == "atomic":
            self.expect("<")
            e = self.parse_type()
            self.expect(">")
            return ("atomic", e)
        if name == "array":
            self.expect("<")
            e = self.parse_type()
            n = None
            if self.accept(","):
                n = int(self.next()[1].rstrip("iu"))
            self.expect(">")
            return ("array", e, n)
        return (name,)

    def attributes(self):
        attrs = {}
        while self.accept("@"):
            name = self.ident()
            args = []
            if self.accept("("):
                while not self.accept(")"):
                    args.append(self.next()[1])
                    self.accept(",")
            attrs[name] = args
        return attrs

    def module(self):
        decls = []
        while self.peek()[0] != "eof":
            attrs = self.attributes()
            kw = self.ident()
            if kw == "struct":
                name = self.ident()
                self.expect("{")
                fields = []
                while not self.accept("}"):
                    self.attributes()
                    fname = self.ident()
                    self.expect(":")
                    fields.append((fname, self.parse_type()))
                    self.accept(",")
                self.accept(";")
                decls.append(("struct", name, fields))
            elif kw == "override":
                name = self.ident()
                self.expect(":")
                ty = self.parse_type()
                init = None
                if self.accept("="):
                    init = self.expr()
                self.expect(";")
                decls.append(("override", name, ty, init))
            elif kw == "var":
                space = None
                if self.accept("<"):
                    space = [self.ident()]
                    while self.accept(","):
                        space.append(self.ident())
                    self.expect(">")
                name = self.ident()
                self.expect(":")
                ty = self.parse_type()
                self.expect(";")
                decls.append(("global", name, ty, space, attrs))
            elif kw == "fn":
                name = self.ident()
                self.expect("(")
                params = []
                while not self.accept(")"):
                    pattrs = self.attributes()
                    pname = self.ident()
                    self.expect(":")
                    params.append((pname, self.parse_type(), pattrs))
                    self.accept(",")
                ret = None
                if self.accept("->"):
                    self.attributes()  # @location / @builtin of an entry point's result
                    ret = self.parse_type()
                body = self.block()
                decls.append(("fn", name, params, ret, body, attrs))
            else:
                raise SyntaxError(f"unexpected {kw}")
        return decls

    def block(self):
        self.expect("{")
        stmts = []
        while not self.accept("}"):
            stmts.append(self.statement())
        return stmts

    def statement(self):
        t = self.peek()
        if t[1] == "{":
            return ("block", self.block())
        if t[1] == "if":
            self.next()
            self.expect("(")
            c = self.expr()
            self.expect(")")
            then = self.block()
            els = None
            if self.accept("else"):
                if self.peek()[1] == "if":
                    els = [self.statement()]
                else:
                    els = self.block()
            return ("if", c, then, els)
        if t[1] == "for":
            self.next()
            self.expect("(")
            init = self.simple_statement()
            self.expect(";")
            cond = self.expr()
            self.expect(";")
            upd = self.simple_statement()
            self.expect(")")
            body = self.block()
            return ("for", init, cond, upd, body)
        if t[1] in ("continue", "break", "discard"):
            self.next()
            self.expect(";")
            return (t[1],)
        if t[1] == "return":
            self.next()
            e = None
            if self.peek()[1] != ";":
                e = self.expr()
            self.expect(";")
            return ("return", e)
        s = self.simple_statement()
        self.expect(";")
        return s

    def simple_statement(self):
        t = self.peek()
        if t[1] in ("var", "let", "const"):
            self.next()
            name = self.ident()
            ty = None
            if self.accept(":"):
                ty = self.parse_type()
            init = None
            if self.accept("="):
                init = self.expr()
            return ("decl", t[1], name, ty, init)
        lhs = self.expr()
        op = self.peek()[1]
        if op in ("=", "+=", "-=", "*=", "/=", "%="):
            self.next()
            rhs = self.expr()
            return ("assign", op, lhs, rhs)
        if op in ("++", "--"):
            self.next()
            return ("assign", "+=" if op == "++" else "-=", lhs, ("lit", "1", "absint"))
        return ("exprstmt", lhs)

    # expressions (precedence climbing)
    BIN = [("||",), ("&&",), ("|",), ("^",), ("&",), ("==", "!="), ("<", ">", "<=", ">="),
           ("+", "-"), ("*", "/", "%")]

    def expr(self, level=0):
        if level == len(self.BIN):
            return self.unary()
        lhs = self.expr(level + 1)
        while self.peek()[1] in self.BIN[level] and self.peek()[0] == "op":
            op = self.next()[1]
            rhs = self.expr(level + 1)
            lhs = ("bin", op, lhs, rhs)
        return lhs

    def unary(self):
        t = self.peek()
        if t[0] == "op" and t[1] in ("-", "!", "&", "*"):
            self.next()
            return ("un", t[1], self.unary())
        return self.postfix(self.primary())

    def primary(self):
        t = self.next()
        if t[0] == "num":
            s = t[1]
            if s.endswith("f"):
                return ("lit", s[:-1], "f32")
            if s.endswith("i"):
                return ("lit", s[:-1], "i32")
            if s.endswith("u"):
                return ("lit", s[:-1], "u32")
            if "." in s or "e" in s or "E" in s:
                return ("lit", s, "absfloat")
            return ("lit", s, "absint")
        if t[1] == "(":
            e = self.expr()
            self.expect(")")
            return e
        if t[0] == "id":
            name = t[1]
            if name in ("true", "false"):
                return ("lit", name, "bool")
            # templated constructor, e.g. vec3<f32>(...)
            if self.peek()[1] == "<" and name in ("vec2", "vec3", "vec4", "array", "mat3x3"):
                self.i -= 1
                ty = self.parse_type()
                self.expect("(")
                return ("call", ty, self.args())
            if self.peek()[1] == "(":
                self.next()
                return ("call", name, self.args())
            return ("ident", name)
        raise SyntaxError(f"unexpected token {t}")

    def args(self):
        out = []
        while not self.accept(")"):
            out.append(self.expr())
            self.accept(",")
        return out

    def postfix(self, e):
        while True:
            if self.accept("."):
                e = ("member", e, self.ident())
            elif self.accept("["):
                idx = self.expr()
                self.expect("]")
                e = ("index", e, idx)
            else:
                return e


# --------------------------------------------------------------------------
# compiler: typed AST -> Python closures
# --------------------------------------------------------------------------

class ReturnSignal(Exception):
    def __init__(self, value):
        self.value = value


class ContinueSignal(Exception):
    pass


class BreakSignal(Exception):
    pass


class DiscardSignal(Exception):
    """A fragment invocation executed `discard`: its entry point returns the
    DISCARDED marker instead of a value."""


DISCARDED = "discarded"


SWZ = {"x": 0, "y": 1, "z": 2, "w": 3, "r": 0, "g": 1, "b": 2, "a": 3}

# exp(x) for f32 x; a fixture generator installs the project's restatement
EXP_F32 = lambda x: np.exp(np.float32(x))  # noqa: E731
# pow(x, y) when installed (the renderer's restatement), else pow(x, 5.0) as a
# product chain and other exponents through float arithmetic
POW_F32 = None
# cube-map lookup of textureSampleLevel, installed by a fixture generator
CUBE_SAMPLE = None


class Module:
    def __init__(self, src: str, overrides: dict):
        self.decls = Parser(src).module()
        self.structs = {}
        self.globals = {}      # name -> type
        self.spaces = {}
        self.funcs = {}
        self.consts = {}
        self.oob = 0
        self._oob_last = None  # (array, index) of the access just before, if out of range
        for d in self.decls:
            if d[0] == "struct":
                self.structs[d[1]] = T("struct", fields=[(f, self.resolve(ty)) for f, ty in d[2]],
                                       name=d[1])
        for d in self.decls:
            if d[0] == "override":
                ty = self.resolve(d[2])
                if d[1] not in overrides:
                    raise KeyError(f"override {d[1]} not provided")
                self.consts[d[1]] = (ty, convert(overrides[d[1]], TABSF, ty))
            elif d[0] == "global":
                self.globals[d[1]] = self.resolve(d[2])
                self.spaces[d[1]] = d[3]
        for d in self.decls:
            if d[0] == "fn":
                self.funcs[d[1]] = d
        self.compiled = {}

    def resolve(self, ty):
        k = ty[0]
        if k in ("f32", "i32", "u32", "bool"):
            return {"f32": TF32, "i32": TI32, "u32": TU32, "bool": TBOOL}[k]
        if k == "vec":
            return vec(self.resolve(ty[2]), ty[1])
        if k == "mat":
            return mat(self.resolve(ty[2]), ty[1])
        if k == "atomic":
            return T("atomic", self.resolve(ty[1]))
        if k == "array":
            return T("array", self.resolve(ty[1]), ty[2] or 0)
        if k in ("texture", "texture_cube"):
            return T(k, self.resolve(ty[1]))
        if k == "sampler":
            return T("sampler")
        if k in self.structs:
            return self.structs[k]
        raise TypeError(f"unknown type {ty}")

    # ---- entry point ------------------------------------------------------
    def count_oob(self, arr, i):
        """Counts out-of-range element accesses once per visit: consecutive
        accesses of one invocation to the same element (a stencil cell's
        four atomics or three field reads) are one, as in the C oracle."""
        key = (id(arr), i)
        if key != self._oob_last:
            self.oob += 1
            self._oob_last = key

    def entry(self, name):
        d = self.funcs[name]
        fn = self.compile_fn(d)
        return fn

    def compile_fn(self, d):
        name = d[1]
        if name in self.compiled:
            return self.compiled[name]
        params = [(p[0], self.resolve(p[1])) for p in d[2]]
        ret = self.resolve(d[3]) if d[3] else None
        scope = {p: t for p, t in params}
        body = self.compile_block(d[4], dict(scope), ret)

        def run(buffers, *args):
            env = {"__buffers__": buffers}
            for (p, _), a in zip(params, args):
                env[p] = a
            try:
                body(env)
            except ReturnSignal as r:
                return r.value
            except DiscardSignal:
                return DISCARDED
            return None

        self.compiled[name] = (run, ret, params)
        return self.compiled[name]

    def compile_block(self, stmts, scope, ret):
        parts = [self.compile_stmt(s, scope, ret) for s in stmts]

        def run(env):
            for p in parts:
                p(env)
        return run

    def compile_stmt(self, s, scope, ret):
        k = s[0]
        if k == "block":
            return self.compile_block(s[1], dict(scope), ret)
        if k == "decl":
            _, kind, name, ty, init = s
            if init is not None:
                ev, et = self.compile_expr(init, scope)
                if ty is not None:
                    target = self.resolve(ty)
                    ev = self.coerce(ev, et, target)
                else:
                    target = self.concretize(et)
                    ev = self.coerce(ev, et, target)
            else:
                target = self.resolve(ty)
                zv = zero_value(target)
                ev = (lambda env, zv=zv: _copy(zv))
            scope[name] = target

            def run(env, ev=ev, name=name):
                env[name] = _copy(ev(env))
            return run
        if k == "assign":
            _, op, lhs, rhs = s
            getter, setter, lt = self.compile_lvalue(lhs, scope)
            rv, rt = self.compile_expr(rhs, scope)
            if op == "=":
                rv = self.coerce(rv, rt, lt)

                def run(env):
                    setter(env, rv(env))
                return run
            binop = op[0]
            f, res_t = self.binary_fn(binop, lt, rt)

            def run(env):
                setter(env, f(getter(env), rv(env)))
            return run
        if k == "exprstmt":
            ev, _ = self.compile_expr(s[1], scope)
            return lambda env: ev(env)
        if k == "if":
            c, _ = self.compile_expr(s[1], scope)
            then = self.compile_block(s[2], dict(scope), ret)
            els = self.compile_block(s[3], dict(scope), ret) if s[3] else None

            def run(env):
                if c(env):
                    then(env)
                elif els is not None:
                    els(env)
            return run
        if k == "for":
            inner = dict(scope)
            init = self.compile_stmt(s[1], inner, ret)
            cond, _ = self.compile_expr(s[2], inner)
            upd = self.compile_stmt(s[3], inner, ret)
            body = self.compile_block(s[4], dict(inner), ret)

            def run(env):
                init(env)
                while cond(env):
                    try:
                        body(env)
                    except ContinueSignal:
                        pass
                    except BreakSignal:
                        break
                    upd(env)
            return run
        if k == "continue":
            def run(env):
                raise ContinueSignal()
            return run
        if k == "break":
            def run(env):
                raise BreakSignal()
            return run
        if k == "discard":
            def run(env):
                raise DiscardSignal()
            return run
        if k == "return":
            if s[1] is None:
                def run(env):
                    raise ReturnSignal(None)
                return run
            ev, et = self.compile_expr(s[1], scope)
            ev = self.coerce(ev, et, ret)

            def run(env):
                raise ReturnSignal(ev(env))
            return run
        raise SyntaxError(f"statement {k}")

    def concretize(self, t):
        if t.kind == "absint":
            return TI32
        if t.kind == "absfloat":
            return TF32
        if t.kind == "vec" and is_abstract(t.elem):
            return vec(self.concretize(t.elem), t.n)
        return t

    def coerce(self, ev, et, target):
        if target is None:
            return ev
        if target.kind == "atomic":
            target = target.elem
        if is_abstract(et) or (et.kind == "vec" and is_abstract(et.elem)):
            return lambda env: convert(ev(env), et, target)
        return ev

    # ---- lvalues -----------------------------------------------------------
    def compile_lvalue(self, e, scope):
        k = e[0]
        if k == "un" and e[1] == "&":
            return self.compile_lvalue(e[2], scope)
        if k == "ident":
            name = e[1]
            if name in scope:
                t = scope[name]
                return (lambda env: env[name]), (lambda env, v: env.__setitem__(name, v)), t
            if name in self.globals:
                t = self.globals[name]
                return ((lambda env: env["__buffers__"][name]),
                        (lambda env, v: env["__buffers__"].__setitem__(name, v)), t)
            raise NameError(name)
        if k == "index":
            bget, bset, bt = self.compile_lvalue(e[1], scope)
            iv, it = self.compile_expr(e[2], scope)
            if bt.kind == "array":
                et = bt.elem

                def get(env):
                    arr = bget(env)
                    i = int(iv(env))
                    if 0 <= i < len(arr):
                        self._oob_last = None
                        return arr[i]
                    self.count_oob(arr, i)
                    return zero_value(et)

                def setv(env, v):
                    arr = bget(env)
                    i = int(iv(env))
                    if 0 <= i < len(arr):
                        self._oob_last = None
                        arr[i] = v
                    else:
                        self.count_oob(arr, i)
                return get, setv, et
            if bt.kind in ("vec", "mat"):
                et = bt.elem if bt.kind == "vec" else vec(bt.elem, bt.n)

                def get(env):
                    return bget(env)[int(iv(env))]

                def setv(env, v):
                    cur = list(bget(env))
                    cur[int(iv(env))] = v
                    bset(env, tuple(cur))
                return get, setv, et
        if k == "member":
            bget, bset, bt = self.compile_lvalue(e[1], scope)
            f = e[2]
            if bt.kind == "struct":
                ft = dict(bt.fields)[f]

                def get(env):
                    return bget(env)[f]

                def setv(env, v):
                    rec = bget(env)
                    if isinstance(rec, dict):
                        rec[f] = v
                return get, setv, ft
            if bt.kind == "vec":
                if len(f) > 1:  # a multi-component swizzle is read as a value
                    raise SyntaxError("swizzle")
                c = SWZ[f]

                def get(env):
                    return bget(env)[c]

                def setv(env, v):
                    cur = list(bget(env))
                    cur[c] = v
                    bset(env, tuple(cur))
                return get, setv, bt.elem
        raise SyntaxError(f"not an lvalue: {e}")

    # ---- expressions -------------------------------------------------------
    def compile_expr(self, e, scope):
        k = e[0]
        if k == "lit":
            s, kind = e[1], e[2]
            if kind == "f32":
                v = F32(float(s))
                return (lambda env: v), TF32
            if kind == "i32":
                v = wrap32(int(s))
                return (lambda env: v), TI32
            if kind == "u32":
                v = int(s) & 0xFFFFFFFF
                return (lambda env: v), TU32
            if kind == "bool":
                v = s == "true"
                return (lambda env: v), TBOOL
            if kind == "absfloat":
                v = float(s)
                return (lambda env: v), TABSF
            v = int(s)
            return (lambda env: v), TABSI
        if k == "ident":
            name = e[1]
            if name in scope:
                t = scope[name]
                return (lambda env: env[name]), t
            if name in self.consts:
                t, v = self.consts[name]
                return (lambda env: v), t
            if name in self.globals:
                t = self.globals[name]
                return (lambda env: env["__buffers__"][name]), t
            raise NameError(name)
        if k in ("index", "member"):
            # rvalue access through the lvalue machinery, copying the result
            get, _, t = self.compile_lvalue_rv(e, scope)
            return (lambda env: get(env)), t
        if k == "un":
            op = e[1]
            if op == "&":
                get, setv, t = self.compile_lvalue(e[2], scope)
                return (lambda env: (get, setv)), T("ptr", t)
            ev, et = self.compile_expr(e[2], scope)
            if op == "-":
                return (lambda env: _neg(ev(env), et)), et
            if op == "!":
                return (lambda env: not ev(env)), TBOOL
        if k == "bin":
            op = e[1]
            lv, lt = self.compile_expr(e[2], scope)
            rv, rt = self.compile_expr(e[3], scope)
            if op in ("&&", "||"):
                if op == "&&":
                    return (lambda env: bool(lv(env)) and bool(rv(env))), TBOOL
                return (lambda env: bool(lv(env)) or bool(rv(env))), TBOOL
            f, t = self.binary_fn(op, lt, rt)
            return (lambda env: f(lv(env), rv(env))), t
        if k == "call":
            return self.compile_call(e[1], e[2], scope)
        raise SyntaxError(f"expression {e}")

    def compile_lvalue_rv(self, e, scope):
        # rvalue member/index on an arbitrary expression (e.g. weights[gx].x)
        try:
            return self.compile_lvalue(e, scope)
        except (SyntaxError, NameError):
            pass
        base_v, bt = self.compile_expr(e[1], scope)
        if e[0] == "member":
            if bt.kind == "vec":
                if len(e[2]) > 1:
                    cs = [SWZ[ch] for ch in e[2]]
                    return ((lambda env: tuple(base_v(env)[c] for c in cs)), None,
                            vec(bt.elem, len(cs)))
                c = SWZ[e[2]]
                return (lambda env: base_v(env)[c]), None, bt.elem
            ft = dict(bt.fields)[e[2]]
            return (lambda env: base_v(env)[e[2]]), None, ft
        iv, _ = self.compile_expr(e[2], scope)
        et = bt.elem if bt.kind in ("vec", "array") else vec(bt.elem, bt.n)
        return (lambda env: base_v(env)[int(iv(env))]), None, et

    def binary_fn(self, op, lt, rt):
        # abstract folding / conversion
        if is_abstract(lt) and is_abstract(rt):
            t = TABSF if "absfloat" in (lt.kind, rt.kind) else TABSI
            return (lambda a, b: _abs_op(op, a, b, t)), (TBOOL if op in CMP else t)
        if is_abstract(lt):
            st = scalar_of(rt)
            f, t = self.binary_fn(op, st, rt)
            return (lambda a, b: f(convert(a, lt, st), b)), t
        if is_abstract(rt):
            st = scalar_of(lt)
            f, t = self.binary_fn(op, lt, st)
            return (lambda a, b: f(a, convert(b, rt, st))), t
        if lt.kind == "atomic":
            lt = lt.elem
        if rt.kind == "atomic":
            rt = rt.elem
        if op in CMP:
            return (lambda a, b: _cmp(op, a, b)), TBOOL
        lk, rk = lt.kind, rt.kind
        if lk in ("f32", "i32", "u32") and rk == lk:
            return (lambda a, b: _sc(op, a, b, lk)), lt
        if lk == "vec" and rk == "vec":
            sk = lt.elem.kind
            return (lambda a, b: tuple(_sc(op, x, y, sk) for x, y in zip(a, b))), lt
        if lk == "vec" and rk in ("f32", "i32", "u32"):
            sk = rk
            return (lambda a, b: tuple(_sc(op, x, b, sk) for x in a)), lt
        if lk in ("f32", "i32", "u32") and rk == "vec":
            sk = lk
            return (lambda a, b: tuple(_sc(op, a, y, sk) for y in b)), rt
        if lk == "mat" and rk == "vec" and op == "*":
            return (lambda m, v: _matvec(m, v)), rt
        if lk == "mat" and rk == "f32" and op == "*":
            return (lambda m, s: tuple(tuple(x * s for x in col) for col in m)), lt
        if lk == "f32" and rk == "mat" and op == "*":
            return (lambda s, m: tuple(tuple(s * x for x in col) for col in m)), rt
        if lk == "mat" and rk == "mat" and op in ("+", "-"):
            return (lambda a, b: tuple(tuple(_sc(op, x, y, "f32") for x, y in zip(ca, cb))
                                       for ca, cb in zip(a, b))), lt
        raise TypeError(f"no operator {lt} {op} {rt}")

    def compile_call(self, callee, args, scope):
        if isinstance(callee, tuple):  # templated type constructor
            return self.construct(self.resolve(callee), args, scope)
        name = callee
        ctor = {"vec3f": vec(TF32), "vec2f": vec(TF32, 2), "vec4f": vec(TF32, 4),
                "vec3i": vec(TI32), "vec3u": vec(TU32), "vec2i": vec(TI32, 2),
                "vec2u": vec(TU32, 2), "vec4i": vec(TI32, 4), "vec4u": vec(TU32, 4),
                "mat3x3f": mat(TF32), "f32": TF32, "i32": TI32, "u32": TU32}
        if name in ctor:
            return self.construct(ctor[name], args, scope)
        if name in self.structs:
            st = self.structs[name]
            fields = [(f, self.coerce(*self.compile_expr(a, scope), ft))
                      for (f, ft), a in zip(st.fields, args)]
            return (lambda env: {f: _copy(ev(env)) for f, ev in fields}), st
        evs = [self.compile_expr(a, scope) for a in args]
        if name in ("vec2", "vec3", "vec4"):
            # element type inferred from the components; an abstract float
            # vector concretises to an f32 vector, an abstract int one to i32
            # (every abstract value these shaders build is exact in f32)
            n = int(name[3])
            kinds = {scalar_of(t).kind for _, t in evs}
            if kinds & {"f32", "absfloat"}:
                return self.construct(vec(TF32, n), args, scope)
            if "u32" in kinds:
                return self.construct(vec(TU32, n), args, scope)
            return self.construct(vec(TI32, n), args, scope)
        if name == "array":
            # array(e0, e1, ...): the elements' (concretised) common type
            et = evs[0][1]
            if is_abstract(et) or (et.kind == "vec" and is_abstract(et.elem)):
                et = self.concretize(et)
            conv = [self.coerce(v, t, et) for v, t in evs]
            return (lambda env: [c(env) for c in conv]), T("array", et, len(conv))
        if name == "abs":
            (v, t), = evs
            if t.kind == "vec":
                return (lambda env: tuple(_cast(abs(x), t.elem) for x in v(env))), t
            if is_abstract(t):
                return (lambda env: abs(v(env))), t
            return (lambda env: _cast(abs(v(env)), t)), t
        if name == "exp":
            # WGSL leaves exp's precision to the implementation: the project's
            # restatement is used wherever it is installed (EXP_F32)
            (v, t), = evs
            if t.kind == "vec":
                return (lambda env: tuple(F32(EXP_F32(F32(x))) for x in v(env))), t
            v = self.coerce(v, t, TF32)
            return (lambda env: F32(EXP_F32(F32(v(env))))), TF32
        if name == "cross":
            (a, at), (b, bt) = evs

            def run(env):
                x, y = a(env), b(env)
                return (F32(F32(x[1] * y[2]) - F32(x[2] * y[1])),
                        F32(F32(x[2] * y[0]) - F32(x[0] * y[2])),
                        F32(F32(x[0] * y[1]) - F32(x[1] * y[0])))
            return run, at
        if name == "reflect":
            # e1 - 2 * dot(e2, e1) * e2
            (a, at), (b, bt) = evs

            def run(env):
                e1, e2 = a(env), b(env)
                k = F32(F32(2.0) * _dot(e2, e1))
                return tuple(F32(F32(x) - F32(k * F32(n))) for x, n in zip(e1, e2))
            return run, at
        if name == "mix":
            # e1 * (1 - e3) + e2 * e3, e3 a scalar or a vector
            (a, at), (b, bt), (c, ct) = evs
            c = self.coerce(c, ct, at.elem if ct.kind != "vec" else ct)

            def run(env):
                e1, e2, e3 = a(env), b(env), c(env)
                ts = e3 if isinstance(e3, tuple) else (e3,) * len(e1)
                return tuple(F32(F32(x * F32(F32(1.0) - t)) + F32(y * t))
                             for x, y, t in zip(e1, e2, ts))
            return run, at
        if name == "textureSampleLevel":
            # the sampling unit's filtering is not shader arithmetic: a fixture
            # generator installs it (CUBE_SAMPLE(texture, direction) -> rgb)
            (tv, tt), _s, (dv, dt_), _lvl = evs

            def run(env):
                r, g, b_ = CUBE_SAMPLE(tv(env), dv(env))
                return (F32(r), F32(g), F32(b_), F32(1.0))
            return run, vec(TF32, 4)
        if name == "textureLoad":
            # a single-channel texture as an (H, W) float32 array; a texel
            # outside it reads the nearest edge texel (WGSL lets an
            # out-of-bounds load return any texel within bounds)
            (tv, tt), (cv, ct), _level = evs

            def run(env):
                img = tv(env)
                x, y = (int(c) for c in cv(env))
                h, w = img.shape
                x = min(max(x, 0), w - 1)
                y = min(max(y, 0), h - 1)
                return (F32(img[y, x]), F32(0.0), F32(0.0), F32(1.0))
            return run, vec(TF32, 4)
        if name == "sqrt":
            (v, t), = evs
            if t.kind == "vec":
                return (lambda env: tuple(F32(np.sqrt(F32(x))) for x in v(env))), t
            if is_abstract(t):
                return (lambda env: float(np.sqrt(v(env)))), t
            return (lambda env: F32(np.sqrt(F32(v(env))))), t
        if name == "dot":
            # ((x0*y0 + x1*y1) + x2*y2), every product and sum rounded to f32
            (a, at), (b, bt) = evs

            def run(env):
                return _dot(a(env), b(env))
            return run, at.elem
        if name == "normalize":
            # v / sqrt(dot(v, v)) component by component (WGSL leaves the
            # precision to the implementation; the C oracle does the same)
            (v, t), = evs

            def run(env):
                x = v(env)
                n = F32(np.sqrt(_dot(x, x)))
                return tuple(F32(F32(c) / n) for c in x)
            return run, t
        if name == "atomicAdd":
            (pv, pt), (vv, vt) = evs
            target = pt.elem if pt.kind == "ptr" else pt
            st = target.elem if target.kind == "atomic" else target
            vv2 = self.coerce(vv, vt, st)

            def run(env):
                get, setv = pv(env)
                old = get(env)
                setv(env, wrap32(old + vv2(env)) if st.kind == "i32" else (old + vv2(env)) & 0xFFFFFFFF)
                return old
            return run, st
        if name == "arrayLength":
            (pv, pt), = evs
            return (lambda env: len(pv(env)[0](env))), TU32
        if name in ("floor", "ceil"):
            (v, t), = evs
            fn = np.floor if name == "floor" else np.ceil
            if t.kind == "vec":
                return (lambda env: tuple(F32(fn(x)) for x in v(env))), t
            if is_abstract(t):
                return (lambda env: float(fn(v(env)))), t
            return (lambda env: F32(fn(v(env)))), t
        if name == "transpose":
            (v, t), = evs
            return (lambda env: _transpose(v(env))), t
        if name in ("max", "min"):
            (a, at), (b, bt) = evs
            t = at if not is_abstract(at) else bt
            a = self.coerce(a, at, scalar_of(t))
            b = self.coerce(b, bt, scalar_of(t))
            f = _wmax if name == "max" else _wmin
            return (lambda env: f(a(env), b(env))), t
        if name == "clamp":
            (e_, et), (lo, lt), (hi, ht) = evs
            t = et
            lo = self.coerce(lo, lt, scalar_of(t))
            hi = self.coerce(hi, ht, scalar_of(t))
            return (lambda env: _wmin(_wmax(e_(env), lo(env)), hi(env))), t
        if name == "pow":
            (a, at), (b, bt) = evs
            t = at if not is_abstract(at) else bt
            a = self.coerce(a, at, scalar_of(t))
            b = self.coerce(b, bt, scalar_of(t))
            return (lambda env: (POW_F32 or _pow)(a(env), b(env))), t
        if name in self.funcs:
            run, ret, params = self.compile_fn(self.funcs[name])
            conv = [self.coerce(ev, et, pt) for (ev, et), (_, pt) in zip(evs, params)]
            return (lambda env: run(env["__buffers__"], *[c(env) for c in conv])), ret
        raise NameError(f"unknown function {name}")

    def construct(self, t, args, scope):
        evs = [self.compile_expr(a, scope) for a in args]
        if t.kind in ("f32", "i32", "u32"):
            (v, vt), = evs
            if t.kind == "f32":
                return (lambda env: F32(v(env))), t
            if t.kind == "i32":
                if scalar_of(vt).kind in ("f32", "absfloat"):
                    return (lambda env: f2i(v(env))), t
                return (lambda env: wrap32(int(v(env)))), t
            if scalar_of(vt).kind in ("f32", "absfloat"):
                return (lambda env: f2u(v(env))), t
            return (lambda env: int(v(env)) & 0xFFFFFFFF), t
        if t.kind == "vec":
            st = t.elem
            if len(evs) == 1 and evs[0][1].kind != "vec":
                v, vt = evs[0]
                v = self.coerce(v, vt, st)
                return (lambda env: tuple(_cast(v(env), st) for _ in range(t.n))), t
            if any(vt.kind == "vec" for _, vt in evs):
                # vector components are spread; a single vector of another
                # element type is converted component by component
                parts = []
                for v, vt in evs:
                    if vt.kind == "vec":
                        parts.append((v, vt.n, vt.elem))
                    else:
                        parts.append((self.coerce(v, vt, st), 0, st))

                def conv(x, src):
                    if st.kind == src.kind:
                        return _cast(x, st)
                    if st.kind == "u32":
                        return f2u(x) if src.kind in ("f32", "absfloat") else int(x) & 0xFFFFFFFF
                    if st.kind == "i32":
                        return f2i(x) if src.kind in ("f32", "absfloat") else wrap32(int(x))
                    return F32(x)

                def run(env):
                    out = []
                    for v, n, src in parts:
                        if n:
                            out.extend(conv(x, src) for x in v(env))
                        else:
                            out.append(_cast(v(env), st))
                    return tuple(out)
                return run, t
            comps = [self.coerce(v, vt, st) for v, vt in evs]
            return (lambda env: tuple(_cast(c(env), st) for c in comps)), t
        if t.kind == "mat":
            if len(evs) == t.n:
                cols = [ev for ev, _ in evs]
                return (lambda env: tuple(tuple(c(env)) for c in cols)), t
            comps = [self.coerce(v, vt, t.elem) for v, vt in evs]
            n = t.n
            return (lambda env: tuple(tuple(comps[c * n + r](env) for r in range(n))
                                      for c in range(n))), t
        raise TypeError(f"constructor {t}")


CMP = ("<", ">", "<=", ">=", "==", "!=")


def _dot(x, y):
    acc = F32(F32(x[0]) * F32(y[0]))
    for i in range(1, len(x)):
        acc = F32(acc + F32(F32(x[i]) * F32(y[i])))
    return acc


def _copy(v):
    if isinstance(v, dict):
        return {k: _copy(x) for k, x in v.items()}
    if isinstance(v, list):
        return [_copy(x) for x in v]
    return v


def _cast(x, st):
    if st.kind == "f32":
        return F32(x)
    return x


def _neg(v, t):
    if isinstance(v, tuple):
        return tuple(_neg(x, t) for x in v)
    if isinstance(v, (int,)) and not isinstance(v, bool):
        if t.kind == "i32":
            return wrap32(-v)
        return -v
    if isinstance(v, float) and not isinstance(v, np.floating):
        return -v
    return F32(-v)


def _abs_op(op, a, b, t):
    if op in CMP:
        return _cmp(op, a, b)
    if op == "+":
        return a + b
    if op == "-":
        return a - b
    if op == "*":
        return a * b
    if op == "/":
        return a / b if t.kind == "absfloat" else int(a / b)
    if op == "%":
        return math.fmod(a, b)
    raise TypeError(op)


def _cmp(op, a, b):
    return {"<": a < b, ">": a > b, "<=": a <= b, ">=": a >= b, "==": a == b, "!=": a != b}[op]


def _sc(op, a, b, kind):
    if kind == "f32":
        with np.errstate(all="ignore"):
            if op == "+":
                return F32(a + b)
            if op == "-":
                return F32(a - b)
            if op == "*":
                return F32(a * b)
            if op == "/":
                return F32(F32(a) / F32(b))
            if op == "%":
                return F32(np.fmod(a, b))
    if kind == "i32":
        if op == "+":
            return wrap32(a + b)
        if op == "-":
            return wrap32(a - b)
        if op == "*":
            return wrap32(a * b)
        if op == "/":
            if b == 0:
                return a
            if a == -2**31 and b == -1:
                return a
            q = abs(a) // abs(b)
            return wrap32(q if (a >= 0) == (b >= 0) else -q)
        if op == "%":
            if b == 0:
                return 0
            if a == -2**31 and b == -1:
                return 0
            r = abs(a) % abs(b)
            return wrap32(r if a >= 0 else -r)
    if kind == "u32":
        m = 0xFFFFFFFF
        if op == "+":
            return (a + b) & m
        if op == "-":
            return (a - b) & m
        if op == "*":
            return (a * b) & m
        if op == "/":
            return a if b == 0 else a // b
        if op == "%":
            return 0 if b == 0 else a % b
    raise TypeError(f"{kind} {op}")


def _matvec(m, v):
    out = []
    with np.errstate(all="ignore"):
        for r in range(len(v)):
            acc = F32(m[0][r] * v[0])
            for c in range(1, len(m)):
                acc = F32(acc + F32(m[c][r] * v[c]))
            out.append(acc)
    return tuple(out)


def _transpose(m):
    n = len(m)
    return tuple(tuple(m[r][c] for r in range(n)) for c in range(n))


def _wmax(a, b):
    if a != a:
        return b
    if b != b:
        return a
    return b if a < b else a


def _wmin(a, b):
    if a != a:
        return b
    if b != b:
        return a
    return b if b < a else a


def _pow(a, b):
    with np.errstate(all="ignore"):
        if float(b) == 5.0:
            x2 = F32(a * a)
            x4 = F32(x2 * x2)
            return F32(x4 * a)
        return F32(float(a) ** float(b))


def dispatch(module: Module, entry: str, buffers: dict, invocations: int, workgroup: int = 64):
    """Runs `entry` for global_invocation_id.x in [0, ceil(invocations/64)*64)."""
    run, _, params = module.entry(entry)
    total = -(-invocations // workgroup) * workgroup
    for i in range(total):
        module._oob_last = None
        run(buffers, (i, 0, 0))
