"""Evaluator of the reference's Fortran source text (TEST INFRASTRUCTURE ONLY).

The reference is Fortran 77/90 and no Fortran compiler exists here, so its
code cannot be built.  This module runs the reference's own statements
instead: it reads the .f / .f90 / .F90 files, translates each subroutine and
function (declarations, assignments, IF blocks, DO loops, CALLs, GOTOs to
labels, RETURN, ALLOCATE) into Python, and executes them in complex128 /
float64 arithmetic.  The operator values it produces therefore come from the
reference's formulas as written, not from a restatement, and pin the C oracle
(oracle/asm_impl.inc) and the CUDA assembly.

Only tests/ and the fixture generator under tests/golden/ use it.  It reads
the reference tree at run time (path given by the caller); nothing of the
reference's source is stored in this repository.

Semantics implemented (the subset the hot-path files use):
  * fixed form (.f: comment lines starting with c/C/*/!, continuation in
    column 6, labels in columns 1-5) and free form (.f90/.F90: `!` comments,
    `&` continuation);
  * REAL and DOUBLE PRECISION -> Python float, COMPLEX -> Python complex,
    INTEGER -> int with Fortran truncating division, LOGICAL -> bool;
    assignment converts to the target's declared type (a COMPLEX value stored
    in a REAL keeps its real part, a REAL stored in an INTEGER truncates);
  * integer powers by repeated multiplication (what gfortran emits for
    constant integer exponents);
  * arrays column-major with declared lower bounds; whole-array `=` fills;
  * arguments by reference (copy-in / copy-out for scalars, shared objects
    for arrays);
  * module variables are one global namespace (USE ... ONLY lists are not
    needed to resolve names in the files evaluated here).
The precision is complex128 throughout (SNGL and REAL(..) of a double keep the
double), the precision of the oracle's c128 mode and of the CUDA kernels.
"""
import cmath
import math
import os
import re

# ---------------------------------------------------------------------------
# source reading
# ---------------------------------------------------------------------------


def _strip_comment(s):
    """Removes a trailing `!` comment outside quotes."""
    q = None
    for i, ch in enumerate(s):
        if q:
            if ch == q:
                q = None
        elif ch in "'\"":
            q = ch
        elif ch == "!":
            return s[:i]
    return s


def _lower_outside_strings(s):
    out, q = [], None
    for ch in s:
        if q:
            out.append(ch)
            if ch == q:
                q = None
        elif ch in "'\"":
            q = ch
            out.append(ch)
        else:
            out.append(ch.lower())
    return "".join(out)


def read_statements(path):
    """Returns [(line_number, label, text)] with continuations joined and
    text lower-cased outside string literals."""
    with open(path, errors="replace") as f:
        lines = f.read().split("\n")
    free = not path.lower().endswith(".f")
    stmts = []
    if not free:
        for n, raw in enumerate(lines, 1):
            if not raw.strip() or raw[0] in "cC*!#":
                continue
            raw = raw.replace("\t", "      ")
            lab, cont, body = raw[:5], raw[5:6], _strip_comment(raw[6:])
            if cont not in (" ", "0", "") and lab.strip() == "" and stmts:
                ln, lb, t = stmts[-1]
                stmts[-1] = (ln, lb, t + " " + body.strip())
                continue
            if not body.strip() and not lab.strip():
                continue
            stmts.append((n, lab.strip(), body.strip()))
    else:
        pending = None
        for n, raw in enumerate(lines, 1):
            if raw.lstrip().startswith("#"):
                continue
            s = _strip_comment(raw).rstrip()
            if not s.strip():
                continue
            st = s.strip()
            if pending is not None:
                if st.startswith("&"):
                    st = st[1:]
                pending = (pending[0], pending[1], pending[2] + " " + st)
            else:
                m = re.match(r"^(\d+)\s+(.*)$", st)
                lab, body = (m.group(1), m.group(2)) if m else ("", st)
                pending = (n, lab, body)
            if pending[2].rstrip().endswith("&"):
                pending = (pending[0], pending[1], pending[2].rstrip()[:-1])
                continue
            stmts.append(pending)
            pending = None
    out = []
    for ln, lab, t in stmts:
        t = _lower_outside_strings(t).strip()
        # statements separated by ';' (outside strings) in free form
        if free and ";" in t:
            parts, cur, q = [], "", None
            for ch in t:
                if q:
                    cur += ch
                    if ch == q:
                        q = None
                elif ch in "'\"":
                    q = ch
                    cur += ch
                elif ch == ";":
                    parts.append(cur)
                    cur = ""
                else:
                    cur += ch
            parts.append(cur)
            for i, p in enumerate(parts):
                if p.strip():
                    out.append((ln, lab if i == 0 else "", p.strip()))
        else:
            out.append((ln, lab, t))
    return out


# ---------------------------------------------------------------------------
# expressions
# ---------------------------------------------------------------------------

_DOTOPS = (".eqv.", ".neqv.", ".and.", ".or.", ".not.", ".eq.", ".ne.", ".lt.", ".le.", ".gt.", ".ge.",
           ".true.", ".false.")
_TOK = re.compile(r"\s*(?:(\d+\.\d*(?:[ed][+-]?\d+)?(?:_\w+)?|\d*\.\d+(?:[ed][+-]?\d+)?(?:_\w+)?|\d+[ed][+-]?\d+(?:_\w+)?"
                  r"|\d+(?:_\w+)?)|([a-z_][a-z0-9_]*)|(\*\*|//|==|/=|<=|>=|=>|[-+*/()<>,=:%])|('(?:[^']|'')*'|\"[^\"]*\"))")


_DOTOP_BLANKS = re.compile(r"\.\s*(eqv|neqv|and|or|not|eq|ne|lt|le|gt|ge|true|false)\s*\.")


def tokenize(s):
    # blanks are not significant in fixed form: `. or.` is `.or.`
    s = _DOTOP_BLANKS.sub(lambda m: "." + m.group(1) + ".", s)
    toks, i = [], 0
    while i < len(s):
        if s[i].isspace():
            i += 1
            continue
        if s[i] == ".":
            for op in _DOTOPS:
                if s.startswith(op, i):
                    toks.append(("op", op))
                    i += len(op)
                    break
            else:
                m = _TOK.match(s, i)
                if not m or not m.group(1):
                    raise SyntaxError("cannot tokenize at %r" % s[i:])
                toks.append(("num", m.group(1)))
                i = m.end()
            continue
        m = _TOK.match(s, i)
        if not m or m.end() == i:
            raise SyntaxError("cannot tokenize at %r" % s[i:])
        num, name, op, st = m.groups()
        if num is not None:
            # `1.eq.` : the dot belongs to the operator
            if num.endswith(".") and any(s.startswith(o, m.start(1) + len(num) - 1) for o in _DOTOPS):
                num = num[:-1]
                toks.append(("num", num))
                i = m.start(1) + len(num)
                continue
            toks.append(("num", num))
        elif name is not None:
            toks.append(("name", name))
        elif op is not None:
            toks.append(("op", op))
        else:
            toks.append(("str", st))
        i = m.end()
    return toks


def _num_literal(t):
    t = re.sub(r"_\w+$", "", t)
    if re.fullmatch(r"\d+", t):
        return int(t)
    return float(t.replace("d", "e"))


# AST: ("num", v) ("str", s) ("name", n) ("call", n, [args]) ("un", op, a) ("bin", op, a, b)
#      ("slice", lo, hi) for ':' inside a call argument list
_BP = {".eqv.": 10, ".neqv.": 10, ".or.": 20, ".and.": 30,
       ".eq.": 50, ".ne.": 50, ".lt.": 50, ".le.": 50, ".gt.": 50, ".ge.": 50,
       "==": 50, "/=": 50, "<": 50, "<=": 50, ">": 50, ">=": 50,
       "//": 60, "+": 70, "-": 70, "*": 80, "/": 80, "**": 90}


class _Parser:
    def __init__(self, toks):
        self.t = toks
        self.i = 0

    def peek(self):
        return self.t[self.i] if self.i < len(self.t) else (None, None)

    def take(self, v=None):
        tok = self.peek()
        if v is not None and tok[1] != v:
            raise SyntaxError("expected %r, got %r" % (v, tok))
        self.i += 1
        return tok

    def expr(self, rbp=0):
        kind, v = self.take()
        if kind == "num":
            left = ("num", _num_literal(v))
        elif kind == "str":
            left = ("str", v[1:-1])
        elif kind == "op" and v in (".true.", ".false."):
            left = ("num", v == ".true.")
        elif kind == "op" and v in ("-", "+"):
            left = ("un", v, self.expr(70))
        elif kind == "op" and v == ".not.":
            left = ("un", "not", self.expr(40))
        elif kind == "op" and v == "(":
            a = self.expr()
            if self.peek()[1] == ",":     # complex constant (re, im)
                self.take(",")
                b = self.expr()
                self.take(")")
                left = ("call", "cmplx", [a, b])
            else:
                self.take(")")
                left = a
        elif kind == "name":
            if self.peek()[1] == "(":
                self.take("(")
                args = []
                if self.peek()[1] != ")":
                    while True:
                        args.append(self.arg())
                        if self.peek()[1] == ",":
                            self.take(",")
                            continue
                        break
                self.take(")")
                left = ("call", v, args)
            else:
                left = ("name", v)
        else:
            raise SyntaxError("unexpected %r" % (v,))
        while True:
            kind, v = self.peek()
            if kind != "op" or v not in _BP or _BP[v] <= rbp:
                if not (kind == "op" and v == "**" and _BP[v] > rbp):
                    break
            bp = _BP[v]
            self.take()
            right = self.expr(bp - 1 if v == "**" else bp)
            left = ("bin", v, left, right)
        return left

    def arg(self):
        # array section a:b, keyword argument name=value
        if self.peek()[1] == ":":
            self.take(":")
            hi = None if self.peek()[1] in (",", ")") else self.expr()
            return ("slice", None, hi)
        if self.peek()[0] == "name" and self.i + 1 < len(self.t) and self.t[self.i + 1][1] == "=":
            nm = self.take()[1]
            self.take("=")
            return ("kw", nm, self.expr())
        a = self.expr()
        if self.peek()[1] == ":":
            self.take(":")
            hi = None if self.peek()[1] in (",", ")") else self.expr()
            return ("slice", a, hi)
        return a


def parse_expr(s):
    p = _Parser(tokenize(s))
    e = p.expr()
    if p.i != len(p.t):
        raise SyntaxError("trailing tokens in %r" % s)
    return e


# ---------------------------------------------------------------------------
# runtime support
# ---------------------------------------------------------------------------


class FArray:
    """Column-major array with Fortran lower bounds."""
    __slots__ = ("lo", "ext", "d", "kind")

    def __init__(self, bounds, kind):
        self.lo = [b[0] for b in bounds]
        self.ext = [b[1] - b[0] + 1 for b in bounds]
        n = 1
        for e in self.ext:
            n *= max(e, 0)
        self.kind = kind
        self.d = [_ZERO[kind]] * n

    def _off(self, idx):
        o, m = 0, 1
        for i, l, e in zip(idx, self.lo, self.ext):
            k = int(i) - l
            if k < 0 or k >= e:
                raise IndexError("index %r out of bounds %r" % (idx, list(zip(self.lo, self.ext))))
            o += k * m
            m *= e
        return o

    def g(self, *idx):
        return self.d[self._off(idx)]

    def s(self, idx, v):
        self.d[self._off(idx)] = v

    def fill(self, v):
        self.d = [v] * len(self.d)


_ZERO = {"integer": 0, "real": 0.0, "double": 0.0, "complex": 0j, "logical": False, "character": ""}


def _cv(kind):
    if kind == "integer":
        return lambda x: int(x.real) if isinstance(x, complex) else int(x)
    if kind in ("real", "double"):
        return lambda x: float(x.real) if isinstance(x, complex) else float(x)
    if kind == "complex":
        return complex
    if kind == "logical":
        return bool
    return lambda x: x


CONV = {k: _cv(k) for k in _ZERO}


def _dv(a, b):
    if isinstance(a, int) and isinstance(b, int) and not isinstance(a, bool):
        q = abs(a) // abs(b)
        return q if (a >= 0) == (b >= 0) else -q
    return a / b


def _pw(a, b):
    if isinstance(b, int):
        if b < 0:
            return 1.0 / _pw(a, -b)
        if b == 0:
            return type(a)(1)
        r = None
        x = a
        n = b
        while n:
            if n & 1:
                r = x if r is None else r * x
            n >>= 1
            if n:
                x = x * x
        return r
    return a ** b


def _sign(a, b):
    return abs(a) if b >= 0 else -abs(a)


def _mod(a, b):
    if isinstance(a, int) and isinstance(b, int):
        return a - _dv(a, b) * b
    return math.fmod(a, b)


def _nint(x):
    return int(math.floor(x + 0.5)) if x >= 0 else -int(math.floor(-x + 0.5))


def _sqrt(x):
    return cmath.sqrt(x) if isinstance(x, complex) else math.sqrt(x)


def _exp(x):
    return cmath.exp(x) if isinstance(x, complex) else math.exp(x)


def _real(x, kind=None):
    return float(x.real) if isinstance(x, complex) else float(x)


def _cmplx(a, b=None, kind=None):
    if b is None:
        return complex(a)
    return complex(float(a.real if isinstance(a, complex) else a), float(b.real if isinstance(b, complex) else b))


INTRINSICS = {
    "real": _real, "dble": _real, "sngl": _real, "float": float, "dfloat": float, "dreal": _real,
    "cmplx": _cmplx, "dcmplx": _cmplx,
    "aimag": lambda x: float(complex(x).imag), "dimag": lambda x: float(complex(x).imag),
    "conjg": lambda x: complex(x).conjugate(), "dconjg": lambda x: complex(x).conjugate(),
    "abs": abs, "cabs": abs, "dabs": abs, "iabs": abs,
    "sqrt": _sqrt, "dsqrt": math.sqrt, "csqrt": lambda x: cmath.sqrt(complex(x)),
    "exp": _exp, "dexp": math.exp, "cexp": lambda x: cmath.exp(complex(x)),
    "log": lambda x: cmath.log(x) if isinstance(x, complex) else math.log(x), "alog": math.log, "dlog": math.log,
    "clog": lambda x: cmath.log(complex(x)), "log10": math.log10,
    "sin": lambda x: cmath.sin(x) if isinstance(x, complex) else math.sin(x), "dsin": math.sin,
    "cos": lambda x: cmath.cos(x) if isinstance(x, complex) else math.cos(x), "dcos": math.cos,
    "tan": math.tan, "dtan": math.tan, "asin": math.asin, "dasin": math.asin, "acos": math.acos,
    "dacos": math.acos, "atan": math.atan, "datan": math.atan, "atan2": math.atan2, "datan2": math.atan2,
    "sinh": math.sinh, "cosh": math.cosh, "tanh": math.tanh,
    "int": lambda x, kind=None: int(x.real) if isinstance(x, complex) else int(x), "ifix": int, "idint": int,
    "nint": _nint, "idnint": _nint,
    "max": max, "max0": max, "amax1": max, "dmax1": max, "min": min, "min0": min, "amin1": min, "dmin1": min,
    "mod": _mod, "sign": _sign, "dsign": _sign, "isign": _sign,
    # EPSILON of a default (single-precision) REAL argument, the only use here
    "epsilon": lambda x: 2.0 ** -23,
    "len_trim": lambda s: len(s.rstrip()), "trim": lambda s: s.rstrip(), "char": chr,
}


class _Goto(Exception):
    def __init__(self, label):
        self.label = label


class FortranStop(Exception):
    pass


# ---------------------------------------------------------------------------
# program units
# ---------------------------------------------------------------------------

_TYPES = (("double precision", "double"), ("double complex", "complex"), ("integer", "integer"),
          ("real", "real"), ("complex", "complex"), ("logical", "logical"), ("character", "character"))


def _split_top(s, sep=","):
    """Splits on `sep` at parenthesis depth 0, outside strings."""
    out, cur, depth, q = [], "", 0, None
    for ch in s:
        if q:
            cur += ch
            if ch == q:
                q = None
            continue
        if ch in "'\"":
            q = ch
        elif ch == "(":
            depth += 1
        elif ch == ")":
            depth -= 1
        if ch == sep and depth == 0:
            out.append(cur)
            cur = ""
        else:
            cur += ch
    out.append(cur)
    return [x.strip() for x in out]


class Var:
    __slots__ = ("kind", "dims", "param", "init", "alloc")

    def __init__(self, kind, dims=None, param=False, init=None, alloc=False):
        self.kind, self.dims, self.param, self.init, self.alloc = kind, dims, param, init, alloc


def _parse_decl(text):
    """Type declaration -> (kind, attrs, [(name, dims_src or None, init_src or None)]) or None."""
    for kw, kind in _TYPES:
        if text.startswith(kw) and (len(text) == len(kw) or not (text[len(kw)].isalnum() or text[len(kw)] == "_")):
            rest = text[len(kw):].strip()
            # kind/len selectors: real*8, real(8), character(len=*), character*(*)
            if rest.startswith("*"):
                m = re.match(r"\*\s*(\(\s*\*\s*\)|\d+)", rest)
                if kind == "real" and m and m.group(1) == "8":
                    kind = "double"
                rest = rest[m.end():].strip() if m else rest[1:].strip()
            elif rest.startswith("("):
                depth, j = 0, 0
                for j, ch in enumerate(rest):
                    depth += ch == "("
                    depth -= ch == ")"
                    if depth == 0:
                        break
                rest = rest[j + 1:].strip()
            attrs = {}
            if "::" in rest:
                head, ents = rest.split("::", 1)
                for a in _split_top(head.lstrip(","), ","):
                    if not a:
                        continue
                    m = re.match(r"(\w+)\s*(?:\((.*)\))?$", a)
                    if m:
                        attrs[m.group(1)] = m.group(2)
            else:
                ents = rest
            out = []
            for e in _split_top(ents):
                if not e:
                    continue
                init = None
                if "=" in e and not e.startswith("=") and "=>" not in e:
                    e, init = [x.strip() for x in e.split("=", 1)]
                m = re.match(r"([a-z_][a-z0-9_]*)\s*(?:\((.*)\))?\s*(?:\*\s*\d+)?$", e)
                if not m:
                    raise SyntaxError("declaration entity %r" % e)
                out.append((m.group(1), m.group(2), init))
            return kind, attrs, out
    return None


class Unit:
    def __init__(self, kind, name, args, path):
        self.kind, self.name, self.args, self.path = kind, name, args, path
        self.stmts = []          # (line, label, text) after the header, up to END
        self.vars = {}           # name -> Var (declared)
        self.implicit_none = False
        self.data = []           # (name, values_src)
        self.result_kind = None


class Program:
    """The reference's program units, translated on first call."""

    def __init__(self, root, files):
        self.root = root
        self.units = {}
        self.modvars = {}
        self.G = type("Globals", (), {})()
        self.compiled = {}
        self.code_src = {}
        for f in files:
            self._load(os.path.join(root, f))
        self._init_modules()

    # ---- loading ----
    def _load(self, path):
        stmts = read_statements(path)
        cur = None
        in_iface = 0
        for ln, lab, t in stmts:
            if re.match(r"^(abstract\s+)?interface\b", t):
                in_iface += 1
                continue
            if re.match(r"^end\s*interface\b", t):
                in_iface -= 1
                continue
            if in_iface:
                continue
            m = re.match(r"^(?:(?:recursive|pure|elemental)\s+)*(?:(integer|real|double precision|complex|logical)\s+)?"
                         r"(subroutine|function)\s+([a-z_][a-z0-9_]*)\s*(?:\((.*)\))?\s*(?:result\s*\((\w+)\))?$", t)
            if m and cur is None:
                args = [a.strip() for a in (m.group(4) or "").split(",") if a.strip()]
                cur = Unit(m.group(2), m.group(3), args, path)
                if m.group(1):
                    cur.result_kind = dict(_TYPES).get(m.group(1), m.group(1))
                continue
            m = re.match(r"^module\s+([a-z_][a-z0-9_]*)$", t)
            if m and cur is None:
                cur = Unit("module", m.group(1), [], path)
                continue
            if cur is not None and re.match(r"^end(\s*(subroutine|function|module)(\s+\w+)?)?$", t):
                self.units[cur.name] = cur
                cur = None
                continue
            if cur is not None:
                cur.stmts.append((ln, lab, t))

    def _init_modules(self):
        for u in self.units.values():
            if u.kind != "module":
                continue
            self._scan_decls(u)
            for name, v in u.vars.items():
                self.modvars[name] = v
        for name, v in self.modvars.items():
            if v.param:
                setattr(self.G, "v_" + name, CONV[v.kind](self._const_eval(v.init)))
            elif v.dims is not None and not v.alloc:
                setattr(self.G, "v_" + name, FArray(self._const_bounds(v.dims), v.kind))
            elif v.dims is not None:
                setattr(self.G, "v_" + name, None)
            else:
                setattr(self.G, "v_" + name, _ZERO[v.kind])

    def _const_eval(self, src):
        e = parse_expr(src)
        env = {"_dv": _dv, "_pw": _pw, "_I": INTRINSICS}
        return eval(self._emit_const(e), env)

    def _emit_const(self, e):
        k = e[0]
        if k == "num":
            return repr(e[1])
        if k == "name":
            v = self.modvars.get(e[1])
            if v is None or not v.param:
                raise SyntaxError("non-constant %r" % e[1])
            return repr(getattr(self.G, "v_" + e[1]))
        if k == "un":
            return "(%s%s)" % ("not " if e[1] == "not" else e[1], self._emit_const(e[2]))
        if k == "bin":
            a, b = self._emit_const(e[2]), self._emit_const(e[3])
            return {"**": "_pw(%s,%s)", "/": "_dv(%s,%s)"}.get(e[1], "(%s " + e[1] + " %s)") % (a, b)
        if k == "call":
            return "_I[%r](%s)" % (e[1], ",".join(self._emit_const(a) for a in e[2]))
        raise SyntaxError("constant expression %r" % (e,))

    def _const_bounds(self, dims_src):
        out = []
        for d in _split_top(dims_src):
            if ":" in d:
                lo, hi = d.split(":", 1)
                out.append((self._const_eval(lo), self._const_eval(hi)))
            else:
                out.append((1, self._const_eval(d)))
        return out

    def _scan_decls(self, u):
        """Collects declarations of a unit (types, dims, parameters, DATA)."""
        for ln, lab, t in u.stmts:
            if t == "implicit none":
                u.implicit_none = True
                continue
            d = _parse_decl(t)
            if d is not None:
                kind, attrs, ents = d
                for name, dims, init in ents:
                    if dims is None and "dimension" in attrs:
                        dims = attrs["dimension"]
                    u.vars[name] = Var(kind, dims, "parameter" in attrs, init, "allocatable" in attrs)
                continue
            m = re.match(r"^dimension\s+(.*)$", t)
            if m:
                for e in _split_top(m.group(1)):
                    mm = re.match(r"(\w+)\s*\((.*)\)$", e)
                    v = u.vars.setdefault(mm.group(1), Var(self._implicit(mm.group(1))))
                    v.dims = mm.group(2)
                continue
            m = re.match(r"^parameter\s*\((.*)\)$", t)
            if m:
                for e in _split_top(m.group(1)):
                    nm, val = [x.strip() for x in e.split("=", 1)]
                    v = u.vars.setdefault(nm, Var(self._implicit(nm)))
                    v.param, v.init = True, val
                continue
            m = re.match(r"^data\s+(.*)$", t)
            if m:
                # groups `name-list / value-list /`, values shared out in order
                for names, vals in re.findall(r"\s*,?\s*([^/]+?)\s*/([^/]*)/", m.group(1)):
                    u.data.append(([x.strip() for x in _split_top(names)], vals))

    @staticmethod
    def _implicit(name):
        return "integer" if name[0] in "ijklmn" else "real"

    # ---- translation ----
    def unit_code(self, name):
        if name in self.compiled:
            return self.compiled[name]
        u = self.units[name]
        self._scan_decls(u)
        tr = _Translator(self, u)
        src = tr.translate()
        self.code_src[name] = src
        env = {"_dv": _dv, "_pw": _pw, "_I": INTRINSICS, "G": self.G, "FArray": FArray, "CONV": CONV,
               "_Goto": _Goto, "FortranStop": FortranStop, "P": self}
        exec(compile(src, "<fortran %s:%s>" % (os.path.basename(u.path), name), "exec"), env)
        fn = env["U_" + name]
        self.compiled[name] = fn
        return fn

    def call(self, name, *args):
        """Calls a subroutine; returns the tuple of its arguments after the call."""
        return self.unit_code(name)(*args)

    def run_fragment(self, basename, first, last):
        """Executes the statements on source lines first..last of `basename`
        (with the declarations of the unit that holds them); module variables
        carry the inputs and the results."""
        for u in list(self.units.values()):
            if os.path.basename(u.path) != basename or u.kind == "module":
                continue
            if not any(first <= ln <= last for ln, _, _ in u.stmts):
                continue
            key = "%s__lines_%d_%d" % (u.name, first, last)
            if key not in self.units:
                f = Unit("subroutine", key, [], u.path)
                f.stmts = [s for s in u.stmts if _Translator._is_spec(s[2]) or first <= s[0] <= last]
                # the unit's dummy arguments become locals of the fragment
                self.units[key] = f
            return self.call(key)
        raise KeyError("no unit of %s holds lines %d-%d" % (basename, first, last))

    def get(self, name):
        return getattr(self.G, "v_" + name)

    def set(self, name, value):
        setattr(self.G, "v_" + name, value)

    def alloc(self, name, *extents):
        v = self.modvars[name]
        a = FArray([(1, e) for e in extents], v.kind)
        self.set(name, a)
        return a


class _Translator:
    def __init__(self, prog, unit):
        self.P = prog
        self.u = unit
        self.lines = []
        self.tmp = 0
        self.targets = set()
        self.cycle_labels = []   # per enclosing DO: labels whose statements end its body with no-ops

    # ---- name resolution ----
    def var(self, name):
        """-> (where, Var) with where in {'local', 'global', 'param_local', 'param_global'} or None."""
        u = self.u
        if name in u.vars:
            v = u.vars[name]
            return ("param_local" if v.param else "local"), v
        if name in u.args:
            return "local", Var(self.P._implicit(name))
        if name in self.P.modvars:
            v = self.P.modvars[name]
            return ("param_global" if v.param else "global"), v
        if u.kind == "function" and name == u.name:
            return "local", Var(u.result_kind or self.P._implicit(name))
        return None

    def ref(self, name):
        r = self.var(name)
        if r is None:
            if self.u.implicit_none:
                raise NameError("%s: undeclared name %r" % (self.u.name, name))
            self.u.vars[name] = Var(self.P._implicit(name))
            return "v_" + name
        where, v = r
        if where == "local":
            return "v_" + name
        if where == "param_local":
            return "v_" + name
        return "G.v_" + name

    # ---- expressions ----
    def ex(self, e):
        k = e[0]
        if k == "num":
            return repr(e[1])
        if k == "str":
            return repr(e[1])
        if k == "name":
            return self.ref(e[1])
        if k == "un":
            if e[1] == "not":
                return "(not %s)" % self.ex(e[2])
            return "(%s%s)" % (e[1], self.ex(e[2]))
        if k == "bin":
            op, a, b = e[1], self.ex(e[2]), self.ex(e[3])
            if op == "**":
                return "_pw(%s, %s)" % (a, b)
            if op == "/":
                return "_dv(%s, %s)" % (a, b)
            py = {".eq.": "==", ".ne.": "!=", ".lt.": "<", ".le.": "<=", ".gt.": ">", ".ge.": ">=", "/=": "!=",
                  ".and.": "and", ".or.": "or", ".eqv.": "==", ".neqv.": "!=", "//": "+"}.get(op, op)
            return "(%s %s %s)" % (a, py, b)
        if k == "call":
            name, args = e[1], e[2]
            r = self.var(name)
            if r is not None and r[1].dims is not None:
                if any(a[0] == "slice" for a in args):
                    raise NotImplementedError("array section in an expression: %r" % (e,))
                return "%s.g(%s)" % (self.ref(name), ", ".join(self.ex(a) for a in args))
            if name in self.P.units and self.P.units[name].kind == "function":
                return "P.unit_code(%r)(%s)" % (name, ", ".join(self.ex(a) for a in args))
            if name in INTRINSICS:
                pos = [self.ex(a) for a in args if a[0] != "kw"]
                kws = ["%s=%s" % (a[1], self.ex(a[2])) for a in args if a[0] == "kw"]
                return "_I[%r](%s)" % (name, ", ".join(pos + kws))
            raise NameError("%s: unknown function or array %r" % (self.u.name, name))
        if k == "kw":
            return self.ex(e[2])
        raise SyntaxError("expression %r" % (e,))

    # ---- statements ----
    def emit(self, ind, s):
        self.lines.append("    " * ind + s)

    def assign_code(self, target, value_src):
        """Python statement storing value_src into a Fortran target expression."""
        if target[0] == "name":
            r = self.var(target[1])
            if r is not None and r[1].dims is not None:
                return "%s.fill(CONV[%r](%s))" % (self.ref(target[1]), r[1].kind, value_src)
            kind = r[1].kind if r else self.P._implicit(target[1])
            return "%s = CONV[%r](%s)" % (self.ref(target[1]), kind, value_src)
        if target[0] == "call":
            r = self.var(target[1])
            if r is None or r[1].dims is None:
                raise NameError("%s: assignment to unknown array %r" % (self.u.name, target[1]))
            if all(a[0] == "slice" and a[1] is None and a[2] is None for a in target[2]):
                return "%s.fill(CONV[%r](%s))" % (self.ref(target[1]), r[1].kind, value_src)
            if any(a[0] == "slice" for a in target[2]):
                raise NotImplementedError("partial array section assignment %r" % (target,))
            return "%s.s((%s,), CONV[%r](%s))" % (self.ref(target[1]), ", ".join(self.ex(a) for a in target[2]),
                                                 r[1].kind, value_src)
        raise SyntaxError("assignment target %r" % (target,))

    def translate(self):
        u = self.u
        # goto targets and DO terminal labels
        for ln, lab, t in u.stmts:
            for m in re.finditer(r"\bgo\s*to\s+(\d+)", t):
                self.targets.add(m.group(1))
        args = ["v_" + a for a in u.args]
        self.emit(0, "def U_%s(%s):" % (u.name, ", ".join(args)))
        # locals: zero-initialised scalars, arrays with constant bounds
        for name, v in u.vars.items():
            if name in u.args:
                continue
            if v.param:
                self.emit(1, "v_%s = CONV[%r](%s)" % (name, v.kind, self.ex(parse_expr(v.init))))
        for name, v in u.vars.items():
            if name in u.args or v.param:
                continue
            deferred = v.dims is not None and all(d.strip() == ":" for d in _split_top(v.dims))
            if v.dims is not None and not v.alloc and not deferred and "*" not in v.dims:
                bounds = []
                for d in _split_top(v.dims):
                    if ":" in d:
                        lo, hi = d.split(":", 1)
                        bounds.append("(%s, %s)" % (self.ex(parse_expr(lo)), self.ex(parse_expr(hi))))
                    else:
                        bounds.append("(1, %s)" % self.ex(parse_expr(d)))
                self.emit(1, "v_%s = FArray([%s], %r)" % (name, ", ".join(bounds), v.kind))
            elif v.dims is None:
                self.emit(1, "v_%s = %r" % (name, _ZERO[v.kind]))
            else:
                self.emit(1, "v_%s = None" % name)
        if u.kind == "function" and u.name not in u.vars:
            self.emit(1, "v_%s = %r" % (u.name, _ZERO[u.result_kind or self.P._implicit(u.name)]))
        for names, vals in u.data:
            items = []
            for it in _split_top(vals):
                m = re.match(r"(\d+)\s*\*\s*(.*)$", it)
                if m:
                    items += [m.group(2)] * int(m.group(1))
                else:
                    items.append(it)
            k = 0
            for nm in names:
                v = u.vars[nm]
                if v.dims is not None:
                    n = 1
                    for d in _split_top(v.dims):
                        lo, hi = (d.split(":", 1) if ":" in d else ("1", d))
                        n *= self.P._const_eval(hi) - self.P._const_eval(lo) + 1
                    for i in range(n):
                        self.emit(1, "v_%s.d[%d] = CONV[%r](%s)" % (nm, i, v.kind, self.ex(parse_expr(items[k]))))
                        k += 1
                else:
                    self.emit(1, "v_%s = CONV[%r](%s)" % (nm, v.kind, self.ex(parse_expr(items[k]))))
                    k += 1
            if k != len(items):
                raise SyntaxError("%s: DATA value count %d for %d targets" % (u.name, len(items), k))
        self.ret = ("return (%s,)" % ", ".join(args)) if u.kind == "subroutine" else "return v_" + u.name
        if u.kind == "subroutine" and not args:
            self.ret = "return ()"
        # executable part (forward GOTOs handled per statement list in block())
        body = [(ln, lab, t) for ln, lab, t in u.stmts if not self._is_spec(t)]
        self.block(body, 1)
        self.emit(1, self.ret)
        return "\n".join(self.lines) + "\n"

    @staticmethod
    def _level0(stmts):
        """Indices of the statements that are not inside a construct of the list."""
        out, depth, open_labels = set(), 0, []
        for j, (ln, lab, t) in enumerate(stmts):
            closing = bool(re.match(r"^(end\s*if|end\s*do|end\s*select)$", t)) or (lab and lab in open_labels)
            if depth == 0 and not closing:
                out.add(j)
            m = re.match(r"^do\s+(\d+)", t)
            if m:
                open_labels.append(m.group(1))
                depth += 1
            elif re.match(r"^do\b", t) or (re.match(r"^if\s*\(.*\)\s*then$", t) and
                                            _Translator._split_logical_if(t)[1] == "then") \
                    or re.match(r"^select\s+case", t):
                depth += 1
            elif re.match(r"^(end\s*if|end\s*do|end\s*select)$", t):
                depth -= 1
            if lab and lab in open_labels:
                depth -= open_labels.count(lab)
                open_labels = [x for x in open_labels if x != lab]
        return out

    def _top_level(self, body, stmt):
        depth = 0
        do_labels = []
        for s in body:
            if s is stmt:
                return depth == 0
            t = s[2]
            if re.match(r"^(if\s*\(.*\)\s*then|do\b|select\s+case)", t):
                m = re.match(r"^do\s+(\d+)", t)
                if m:
                    do_labels.append(m.group(1))
                depth += 1
            elif re.match(r"^(end\s*if|end\s*do|enddo|endif|end\s*select)$", t):
                depth -= 1
            if s[1] and s[1] in do_labels:
                depth -= do_labels.count(s[1])
                do_labels = [x for x in do_labels if x != s[1]]
        return depth == 0

    @staticmethod
    def _is_spec(t):
        if _parse_decl(t) is not None and not re.match(r"^(real|integer|complex|logical)\s*\(.*\)\s*=", t):
            # `real(x) = ...` cannot appear; a declaration it is
            return True
        return bool(re.match(r"^(use\b|implicit\b|dimension\b|parameter\s*\(|data\b|save\b|external\b|intrinsic\b|"
                             r"include\b|common\b|format\b|contains\b|equivalence\b)", t))

    def block(self, stmts, ind):
        """A statement list.  Labels in it that a GOTO names split it into
        segments; a GOTO raises _Goto, and the segment list resumes at the
        label's segment (forward jumps: search-loop exits, error sections)."""
        lvl0 = self._level0(stmts)
        cuts = [j for j, st in enumerate(stmts) if j > 0 and j in lvl0 and st[1] and st[1] in self.targets]
        if not cuts:
            i = 0
            while i < len(stmts):
                i = self.stmt(stmts, i, ind)
            return
        bounds = [0] + cuts + [len(stmts)]
        labels = [stmts[c][1] for c in cuts]
        self.tmp += 1
        pc = "_pc%d" % self.tmp
        self.emit(ind, "%s = 0" % pc)
        for k in range(len(bounds) - 1):
            later = {lab: q + 1 for q, lab in enumerate(labels) if q + 1 > k}
            self.emit(ind, "if %s <= %d:" % (pc, k))
            self.emit(ind + 1, "try:")
            n0 = len(self.lines)
            i = bounds[k]
            while i < bounds[k + 1]:
                i = self.stmt(stmts[:bounds[k + 1]], i, ind + 2)
            if len(self.lines) == n0:
                self.emit(ind + 2, "pass")
            self.emit(ind + 1, "except _Goto as _g:")
            self.emit(ind + 2, "if _g.label not in %r: raise" % (later,))
            self.emit(ind + 2, "%s = %r[_g.label]" % (pc, later))

    def _find_block_end(self, stmts, i):
        """For an IF-THEN at i: indices of ELSE IF / ELSE and the END IF."""
        depth, parts = 0, []
        for j in range(i + 1, len(stmts)):
            t = stmts[j][2]
            if re.match(r"^if\s*\(.*\)\s*then$", t):
                depth += 1
            elif re.match(r"^(end\s*if)$", t):
                if depth == 0:
                    return parts, j
                depth -= 1
            elif depth == 0 and re.match(r"^else\s*if\s*\(.*\)\s*then$", t):
                parts.append(j)
            elif depth == 0 and t == "else":
                parts.append(j)
        raise SyntaxError("%s: unterminated IF at line %d" % (self.u.name, stmts[i][0]))

    def _find_do_end(self, stmts, i, label):
        depth = 0
        for j in range(i + 1, len(stmts)):
            t = stmts[j][2]
            if label is None:
                if re.match(r"^do\b(?!\s+\d)", t) and not re.match(r"^do\s+\d", t):
                    depth += 1
                elif re.match(r"^(end\s*do)$", t):
                    if depth == 0:
                        return j
                    depth -= 1
            elif stmts[j][1] == label:
                return j
        raise SyntaxError("%s: unterminated DO at line %d" % (self.u.name, stmts[i][0]))

    def stmt(self, stmts, i, ind):
        ln, lab, t = stmts[i]
        m = re.match(r"^if\s*\((.*)\)\s*then$", t)
        if m and self._balanced_if(t):
            parts, end = self._find_block_end(stmts, i)
            bounds = [i] + parts + [end]
            for k in range(len(bounds) - 1):
                a, b = bounds[k], bounds[k + 1]
                head = stmts[a][2]
                if k == 0:
                    self.emit(ind, "if %s:" % self.ex(parse_expr(self._if_cond(head))))
                elif head == "else":
                    self.emit(ind, "else:")
                else:
                    mm = re.match(r"^else\s*if\s*(\(.*\))\s*then$", head)
                    self.emit(ind, "elif %s:" % self.ex(parse_expr(mm.group(1))))
                n0 = len(self.lines)
                self.block(stmts[a + 1:b], ind + 1)
                if len(self.lines) == n0:
                    self.emit(ind + 1, "pass")
            return end + 1
        m = re.match(r"^do\s+(?:(\d+)\s*,?\s*)?([a-z_]\w*)\s*=\s*(.*)$", t)
        if m:
            label, var, rng = m.group(1), m.group(2), _split_top(m.group(3))
            end = self._find_do_end(stmts, i, label)
            body = stmts[i + 1:end] if label is None else stmts[i + 1:end + 1]
            self.tmp += 1
            k = self.tmp
            a, b = self.ex(parse_expr(rng[0])), self.ex(parse_expr(rng[1]))
            s = self.ex(parse_expr(rng[2])) if len(rng) > 2 else "1"
            v = self.ref(var)
            self.emit(ind, "_a%d = %s; _s%d = %s; _n%d = max(0, _dv(%s - _a%d + _s%d, _s%d))"
                      % (k, a, k, s, k, b, k, k, k))
            self.emit(ind, "for _k%d in range(_n%d):" % (k, k))
            self.emit(ind + 1, "%s = _a%d + _k%d * _s%d" % (v, k, k, k))
            n0 = len(self.lines)
            # a GOTO to a label followed only by CONTINUEs up to the loop end
            # is a CYCLE of this loop
            cyc = set()
            for j in range(len(body) - 1, -1, -1):
                if body[j][2] not in ("continue", "end do", "enddo"):
                    break
                if body[j][1]:
                    cyc.add(body[j][1])
            self.cycle_labels.append(cyc)
            if label is not None and body and body[-1][2] in ("continue", "end do", "enddo"):
                self.block(body[:-1], ind + 1)
            else:
                self.block(body, ind + 1)
            self.cycle_labels.pop()
            if len(self.lines) == n0:
                self.emit(ind + 1, "pass")
            self.emit(ind, "%s = _a%d + _n%d * _s%d" % (v, k, k, k))
            return end + 1
        m = re.match(r"^if\s*\(", t)
        if m:
            cond, rest = self._split_logical_if(t)
            self.emit(ind, "if %s:" % self.ex(parse_expr(cond)))
            self.simple(rest, ind + 1)
            return i + 1
        self.simple(t, ind)
        return i + 1

    def _balanced_if(self, t):
        cond, rest = self._split_logical_if(t)
        return rest.strip() == "then"

    @staticmethod
    def _split_logical_if(t):
        j = t.index("(")
        depth = 0
        for k in range(j, len(t)):
            depth += t[k] == "("
            depth -= t[k] == ")"
            if depth == 0:
                return t[j:k + 1], t[k + 1:].strip()
        raise SyntaxError("unbalanced IF: %r" % t)

    @staticmethod
    def _if_cond(t):
        return _Translator._split_logical_if(t)[0]

    def simple(self, t, ind):
        if t in ("continue", "end do", "enddo"):
            self.emit(ind, "pass")
            return
        if t == "return":
            self.emit(ind, self.ret)
            return
        if t in ("exit",):
            self.emit(ind, "break")
            return
        if t in ("cycle",):
            self.emit(ind, "continue")
            return
        m = re.match(r"^go\s*to\s+(\d+)$", t)
        if m:
            if self.cycle_labels and m.group(1) in self.cycle_labels[-1]:
                self.emit(ind, "continue")
            else:
                self.emit(ind, "raise _Goto(%r)" % m.group(1))
            return
        if re.match(r"^stop\b", t):
            self.emit(ind, "raise FortranStop(%r)" % t)
            return
        if re.match(r"^(write|print|read|open|close|flush)\b", t):
            self.emit(ind, "pass")
            return
        m = re.match(r"^call\s+([a-z_]\w*)\s*(?:\((.*)\))?$", t)
        if m:
            self.call_stmt(m.group(1), m.group(2) or "", ind)
            return
        m = re.match(r"^allocate\s*\((.*)\)$", t)
        if m:
            for e in _split_top(m.group(1)):
                if "=" in e:      # stat=
                    nm, v = [x.strip() for x in e.split("=", 1)]
                    self.emit(ind, self.assign_code(("name", nm), "0"))
                    continue
                mm = re.match(r"(\w+)\s*\((.*)\)$", e)
                r = self.var(mm.group(1))
                bounds = []
                for d in _split_top(mm.group(2)):
                    if ":" in d:
                        lo, hi = d.split(":", 1)
                        bounds.append("(%s, %s)" % (self.ex(parse_expr(lo)), self.ex(parse_expr(hi))))
                    else:
                        bounds.append("(1, %s)" % self.ex(parse_expr(d)))
                self.emit(ind, "%s = FArray([%s], %r)" % (self.ref(mm.group(1)), ", ".join(bounds), r[1].kind))
            return
        if re.match(r"^deallocate\b", t) or re.match(r"^nullify\b", t):
            self.emit(ind, "pass")
            return
        # assignment
        parts = _split_top(t, "=")
        if len(parts) == 2 and not parts[1].startswith(">"):
            target = _Parser(tokenize(parts[0])).expr()
            self.emit(ind, self.assign_code(target, self.ex(parse_expr(parts[1]))))
            return
        raise SyntaxError("%s: unsupported statement %r" % (self.u.name, t))

    def call_stmt(self, name, argsrc, ind):
        args = [a for a in _split_top(argsrc)] if argsrc.strip() else []
        asts = [_Parser(tokenize(a)).arg() for a in args]
        self.tmp += 1
        r = "_r%d" % self.tmp
        if name not in self.P.units:
            raise NameError("%s: CALL of unknown routine %r" % (self.u.name, name))
        self.emit(ind, "%s = P.unit_code(%r)(%s)" % (r, name, ", ".join(self.ex(a) for a in asts)))
        for k, a in enumerate(asts):
            if a[0] == "name":
                rr = self.var(a[1])
                if rr is not None and rr[0] in ("local", "global") and rr[1].dims is None:
                    self.emit(ind, "%s = %s[%d]" % (self.ref(a[1]), r, k))
            elif a[0] == "call":
                rr = self.var(a[1])
                if rr is not None and rr[1].dims is not None and not any(x[0] == "slice" for x in a[2]):
                    self.emit(ind, "%s.s((%s,), %s[%d])" % (self.ref(a[1]), ", ".join(self.ex(x) for x in a[2]),
                                                            r, k))


# ---------------------------------------------------------------------------
# drivers: the reference's own call sequences
# ---------------------------------------------------------------------------

ASSEMBLY_FILES = ("modules.F90", "setcoefs3d.f", "calcwts.f", "fdfd3d.f", "pfdfd3d.f", "pml3d.f", "fixed3d.f",
                  "tpfree.f", "zeroas.f", "asmble.f90", "srgraphs.f", "sparse.f", "modelio.f90", "readini.f90",
                  "dispersion.f", "hetfldsrc.f90", "haskgrn.f", "srcsetup.f", "srcreg.f")


def load_assembly(ref_root):
    return Program(ref_root, ASSEMBLY_FILES)


def reference_pattern(P, nx, ny, nz):
    """srel3d_getsize + srel3d + SPARSE_ADJ2CRS (elwave.f90:112-122):
    1-based irptr (n+1) and jcptr (nnz) as Python lists."""
    r = P.call("srel3d_getsize", nx, ny, nz, 0, 0)
    numvert, nedge = r[3], r[4]
    xadj = FArray([(1, numvert + 1)], "integer")
    adj = FArray([(1, 2 * nedge)], "integer")
    P.call("srel3d", nx, ny, nz, numvert, nedge, xadj, adj)
    nzero = 2 * nedge + numvert
    irptr = FArray([(1, numvert + 1)], "integer")
    jcptr = FArray([(1, nzero)], "integer")
    P.call("sparse_adj2crs", nzero, numvert, xadj, adj, irptr, jcptr)
    return irptr, jcptr


def _set_model(P, nx, ny, nz, vp, vs, rho):
    """vpr, vsr, rho of MODEL_MODULE from [iz, ix, iy] arrays, then lambda and
    mu (and the background copies) by the reference's loop (modelio.f90:78-92)."""
    for nm in ("rho", "rhop", "vpr", "vsr", "mu", "da", "mup", "dap"):
        P.alloc(nm, nz, nx, ny)
    a_vp, a_vs, a_rho = P.get("vpr"), P.get("vsr"), P.get("rho")
    for iy in range(ny):
        for ix in range(nx):
            for iz in range(nz):
                a_vp.s((iz + 1, ix + 1, iy + 1), float(vp[iz, ix, iy]))
                a_vs.s((iz + 1, ix + 1, iy + 1), float(vs[iz, ix, iy]))
                a_rho.s((iz + 1, ix + 1, iy + 1), float(rho[iz, ix, iy]))
    P.run_fragment("modelio.f90", 78, 92)


def _set_grid(P, nx, ny, nz, dx, omega, pmld, fst, usemin, pmlr):
    """Grid, boundary and PML state as readini.f90 sets it: dx = dy = dz,
    freesurf(1) = fst and the other faces false (readini.f90:67-73), pmlr,
    pmld, then ipml and pmlf by the reference's statements (readini.f90:83-84)."""
    P.set("nx", nx); P.set("ny", ny); P.set("nz", nz)
    for d in ("dx", "dy", "dz"):
        P.set(d, float(dx))
    fs = P.get("freesurf")
    fs.fill(False)
    fs.s((1,), bool(fst))
    P.set("usemin", bool(usemin))
    P.set("pmlr", float(pmlr))
    P.set("pmld", float(pmld))
    P.run_fragment("readini.f90", 83, 84)
    P.set("omega", complex(omega))


def reference_hetfldsrc(ref_root, nx, ny, nz, dx, model, background, omega, pmld, fst, usemin, u0, srcfn=1.0,
                        pmlr=1e-3, program=None):
    """Runs HETFLDSRC (hetfldsrc.f90:17-1038): sfld = ((A_bg - A) u0) * srcfn
    with SETCOEFS3D(ibg = 0) on the model and (ibg = 1) on the background.
    u0: dof vector (3 per node, node order z fastest).  The output index of
    hetfldsrc.f90:1020 uses nx*ny for nx*nz, so callers give ny == nz, where
    both agree.  Returns (sfld list, ierr)."""
    P = program or load_assembly(ref_root)
    _set_grid(P, nx, ny, nz, dx, omega, pmld, fst, usemin, pmlr)
    _set_model(P, nx, ny, nz, *background)
    bg = {nm: P.get(nm) for nm in ("rho", "mu", "da")}
    _set_model(P, nx, ny, nz, *model)
    P.set("rhop", bg["rho"]); P.set("mup", bg["mu"]); P.set("dap", bg["da"])
    comps = []
    for c, nm in enumerate(("utbkr", "vtbkr", "wtbkr")):
        a = P.alloc(nm, nz, nx, ny)
        for iy in range(ny):
            for ix in range(nx):
                for iz in range(nz):
                    g = iz + nz * (ix + nx * iy)
                    a.s((iz + 1, ix + 1, iy + 1), complex(u0[3 * g + c]))
        comps.append(a)
    sfld = FArray([(1, 3 * nx * ny * nz)], "complex")
    r = P.call("hetfldsrc", complex(srcfn), sfld, 0, 0, 0)
    return sfld.d, r[-1]


def reference_dispersed_assemble(ref_root, nx, ny, nz, dx, vp, vs, rho, qp, qs, freqbase, omega, pmld, fst,
                                 usemin, pmlr=1e-3, program=None):
    """DISPERSION (dispersion.f:2-114) on the model's lambda and mu at omega,
    then ASMBLE: the operator of an attenuating model.  qp, qs = 1/Q per node."""
    P = program or load_assembly(ref_root)
    _set_grid(P, nx, ny, nz, dx, omega, pmld, fst, usemin, pmlr)
    _set_model(P, nx, ny, nz, vp, vs, rho)
    for nm, arr in (("qp", qp), ("qs", qs)):
        a = P.alloc(nm, nz, nx, ny)
        for iy in range(ny):
            for ix in range(nx):
                for iz in range(nz):
                    a.s((iz + 1, ix + 1, iy + 1), float(arr[iz, ix, iy]))
    P.set("freqbase", float(freqbase))
    P.set("ncom", 0)
    P.call("dispersion")
    irptr, jcptr = reference_pattern(P, nx, ny, nz)
    nzero = len(jcptr.d)
    a = FArray([(1, nzero)], "complex")
    r = P.call("asmble", 6, nzero, nx, ny, nz, irptr, jcptr, a, 0)
    return irptr.d, jcptr.d, a.d, r[-1]


def reference_haskgrn(ref_root, vp1d, vs1d, rh1d, h1d, omega, ain, nz, dz, s_wave=False, zorig=0.0, program=None):
    """HASKGRN (haskgrn.f:31-672) for one incident P (or S) plane wave:
    (ugrn1f, wgrn1f, ierr); the layer velocities double as the discrete ones
    (vp1disc = vp1d, vs1disc = vs1d)."""
    P = program or load_assembly(ref_root)
    nl = len(vp1d)
    P.set("nl", nl); P.set("nz", nz); P.set("dz", float(dz)); P.set("zorig", float(zorig))
    for nm, arr in (("vp1d", vp1d), ("vs1d", vs1d), ("rh1d", rh1d), ("h1d", h1d), ("vp1disc", vp1d),
                    ("vs1disc", vs1d)):
        a = P.alloc(nm, nl)
        for i in range(nl):
            a.s((i + 1,), float(arr[i]))
    P.alloc("ugrn1f", nz)
    P.alloc("wgrn1f", nz)
    P.alloc("ain", 1).s((1,), float(ain))
    P.alloc("srctyp", 1).s((1,), "ps" if s_wave else "pp")
    r = P.call("haskgrn", float(omega), 1, 0)
    return P.get("ugrn1f").d, P.get("wgrn1f").d, r[-1]


def reference_point_source(ref_root, nx, ny, nz, dx, fst, xloc, yloc, zloc, sprd, ireg, sterm=1.0, program=None):
    """SRCSETUP with lsetup = .true. (srcsetup.f:1-214, srcreg.f): the source
    term spread over the grid, swave[iz, ix, iy] as a flat list in node order
    (z fastest); returns (swave, ierr)."""
    P = program or load_assembly(ref_root)
    P.set("nx", nx); P.set("ny", ny); P.set("nz", nz)
    for d in ("dx", "dy", "dz"):
        P.set(d, float(dx))
    fs = P.get("freesurf")
    fs.fill(False)
    fs.s((1,), bool(fst))
    sw = FArray([(1, nz), (1, nx), (1, ny)], "complex")
    r = P.call("srcsetup", True, float(xloc), float(yloc), float(zloc), float(sprd), int(ireg), complex(sterm),
               sw, 0)
    return sw.d, r[-1]


def reference_assemble(ref_root, nx, ny, nz, dx, vp, vs, rho, omega, pmld, fst, usemin, pmlr=1e-3,
                       program=None):
    """Runs the reference's ASMBLE (asmble.f90:1-636) on one grid.

    vp, vs, rho: float arrays indexed [iz-1, ix-1, iy-1] (the reference's
    (nz,nx,ny) order).  The module state is set as readini.f90 and
    modelio.f90 set it (_set_grid, _set_model).  Returns (irptr, jcptr, a,
    ierr, {ipml, pmlf}) with 1-based CSR lists and complex values."""
    P = program or load_assembly(ref_root)
    _set_grid(P, nx, ny, nz, dx, omega, pmld, fst, usemin, pmlr)
    _set_model(P, nx, ny, nz, vp, vs, rho)
    irptr, jcptr = reference_pattern(P, nx, ny, nz)
    nzero = len(jcptr.d)
    a = FArray([(1, nzero)], "complex")
    r = P.call("asmble", 6, nzero, nx, ny, nz, irptr, jcptr, a, 0)
    return irptr.d, jcptr.d, a.d, r[-1], {"ipml": P.get("ipml"), "pmlf": P.get("pmlf")}
