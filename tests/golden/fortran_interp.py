"""An interpreter of the Fortran 77/90 subset that ekman_bl's hot path is
written in.  TEST INFRASTRUCTURE ONLY: it runs the reference's own source
files (read from the reference tree when the fixtures in this directory are
regenerated) so that golden vectors come from the reference's code itself,
not from a restatement of it.  There is no Fortran compiler on the machines
this project builds on; this module stands in for one, for the statements
those files use.

How it works.  Every source file is split into logical statements (fixed
form with DEC tab lines, or free form), grouped into program units (MODULE,
SUBROUTINE, FUNCTION).  A unit is translated into the source of one Python
function the first time it is called, then run by CPython.  Semantics kept:
- storage: every variable has storage of its Fortran type (numpy int32,
  float32, float64, complex64, complex128, bool); arrays are column-major
  with their declared lower bounds; COMMON blocks and EQUIVALENCE groups
  share byte buffers, so storage association works as in Fortran;
- arguments pass by reference; an array element passed to an array dummy
  starts the dummy at that element (sequence association);
- arithmetic follows Fortran's typing: integer division truncates toward
  zero, a REAL literal without a D exponent is a REAL*4 constant, mixed
  operands are converted to the wider kind before the operation, CMPLX
  without KIND yields a single-precision complex;
- DO loops compute their trip count on entry; GO TO targets labels of the
  unit's outermost statement list (or the terminal label of the enclosing
  DO, which acts as CYCLE); STOP raises FortranStop.
Input/output statements are ignored (the harness reads results from the
variables).  Unsupported statements raise NotImplementedError when the
unit containing them is translated.
"""
from __future__ import annotations

import math
import os
import re

import numpy as np


class FortranStop(Exception):
    pass


class _Goto(Exception):
    def __init__(self, label):
        super().__init__(label)
        self.label = label


# ---------------------------------------------------------------------------
# source form
def _split_code_comment(text: str, free: bool):
    """Lowercase outside strings; cut a trailing ! comment."""
    out, q = [], None
    for ch in text:
        if q:
            out.append(ch)
            if ch == q:
                q = None
            continue
        if ch in "'\"":
            q = ch
            out.append(ch)
            continue
        if ch == "!":
            break
        out.append(ch.lower())
    return "".join(out)


def read_statements(path: str, includes: dict[str, str] | None = None):
    """Logical statements of a source file: [(label or None, text, lineno)]."""
    free = path.lower().endswith((".f90", ".f95"))
    with open(path, encoding="latin-1") as f:
        raw = f.read().split("\n")
    return _statements(raw, free, includes or {}, os.path.dirname(path))


def _statements(raw, free, includes, folder):
    stmts = []
    if free:
        buf, start = "", 0
        for n, line in enumerate(raw, 1):
            code = _split_code_comment(line, True).rstrip()
            if not code.strip():
                continue
            s = code.strip()
            if buf and s.startswith("&"):
                s = s[1:]
            if not buf:
                start = n
            if s.endswith("&"):
                buf += s[:-1] + " "
                continue
            buf += s
            _emit(stmts, buf, start, free, includes, folder)
            buf = ""
        if buf:
            _emit(stmts, buf, start, free, includes, folder)
    else:
        cur, start = None, 0
        for n, line in enumerate(raw, 1):
            if not line.strip() or line[0] in "cC*!":
                continue
            line = line.rstrip("\r")
            if line.startswith("\t"):
                body = line[1:]
                if body[:1].isdigit() and body[:1] != "0":
                    cont, label, text = True, "", body[1:]
                else:
                    cont, label, text = False, "", body
            else:
                lab = line[:5]
                if "\t" in lab:  # label then tab
                    i = line.index("\t")
                    lab, text, cont = line[:i], line[i + 1:], False
                else:
                    c6 = line[5:6]
                    cont = c6 not in ("", " ", "0")
                    text = line[6:]
                label = lab.strip()
            text = _split_code_comment(text, False)
            if cont and cur is not None:
                cur[1] += text
                continue
            if cur is not None:
                _emit(stmts, cur[1], cur[2], free, includes, folder, cur[0])
            cur = [label or None, text, n]
        if cur is not None:
            _emit(stmts, cur[1], cur[2], free, includes, folder, cur[0])
    return stmts


def _split_semicolons(text):
    parts, q, buf = [], None, []
    for ch in text:
        if q:
            buf.append(ch)
            if ch == q:
                q = None
            continue
        if ch in "'\"":
            q = ch
        if ch == ";":
            parts.append("".join(buf))
            buf = []
            continue
        buf.append(ch)
    parts.append("".join(buf))
    return [p for p in parts if p.strip()]


def _emit(stmts, text, lineno, free, includes, folder, label=None):
    for part in _split_semicolons(text):
        s = part.strip()
        lab = label
        if free:
            m = re.match(r"^(\d+)\s+(.*)$", s)
            if m:
                lab, s = m.group(1), m.group(2)
        m = re.match(r"^include\s*['\"]([^'\"]+)['\"]\s*$", s)
        if m:
            name = m.group(1)
            if name in includes:
                src = includes[name]
            else:
                with open(os.path.join(folder, name), encoding="latin-1") as f:
                    src = f.read()
            stmts.extend(_statements(src.split("\n"), free, includes, folder))
            continue
        stmts.append((int(lab) if lab else None, s, lineno))
        label = None


# ---------------------------------------------------------------------------
# expressions
_TOKEN = re.compile(r"""
   (?P<ws>\s+)
 | (?P<num>(\d+\.\d*|\.\d+|\d+)([ed][+-]?\d+)?(_\w+)?)
 | (?P<dotop>\.(eq|ne|lt|le|gt|ge|and|or|not|eqv|neqv|true|false)\.)
 | (?P<str>'[^']*'|"[^"]*")
 | (?P<name>[a-z_][a-z0-9_]*)
 | (?P<op>\*\*|//|==|/=|<=|>=|[-+*/()<>,:%=])
""", re.X)


def tokenize(s):
    toks, pos = [], 0
    while pos < len(s):
        m = _TOKEN.match(s, pos)
        if not m:
            raise SyntaxError(f"cannot tokenize {s[pos:]!r} in {s!r}")
        pos = m.end()
        k = m.lastgroup
        if k == "ws":
            continue
        v = m.group(k)
        if k == "num":
            # a number followed by a dotted operator: 1.eq.x -> '1' '.eq.'
            mm = re.match(r"^(\d+)\.(eq|ne|lt|le|gt|ge|and|or|not|eqv|neqv)\.", s[m.start():])
            if mm:
                toks.append(("num", mm.group(1)))
                pos = m.start() + len(mm.group(1))
                continue
        toks.append((k, v))
    return toks


# AST: ('num', text) ('str', text) ('name', id) ('call', id, [args]) ('bin', op, a, b)
# ('un', op, a) ('cplx', re, im) ('range', lo, hi, step) ('kw', name, expr)
class _P:
    PREC = {".eqv.": 1, ".neqv.": 1, ".or.": 2, ".and.": 3, ".not.": 4,
            "==": 5, "/=": 5, "<": 5, "<=": 5, ">": 5, ">=": 5,
            ".eq.": 5, ".ne.": 5, ".lt.": 5, ".le.": 5, ".gt.": 5, ".ge.": 5,
            "//": 6, "+": 7, "-": 7, "*": 8, "/": 8, "**": 10}

    def __init__(self, toks):
        self.t, self.i = toks, 0

    def peek(self, k=0):
        j = self.i + k
        return self.t[j] if j < len(self.t) else (None, None)

    def take(self, v=None):
        tok = self.peek()
        if v is not None and tok[1] != v:
            raise SyntaxError(f"expected {v!r}, got {tok!r}")
        self.i += 1
        return tok

    def expr(self, minp=0):
        k, v = self.peek()
        if v in ("-", "+"):
            self.take()
            a = self.expr(7.5)  # unary minus binds looser than * and **
            a = ("un", v, a)
        elif v == ".not.":
            self.take()
            a = ("un", ".not.", self.expr(4))
        else:
            a = self.primary()
        while True:
            k, v = self.peek()
            if k not in ("op", "dotop") or v not in self.PREC:
                return a
            p = self.PREC[v]
            if p < minp or (p == minp and v != "**"):
                return a
            self.take()
            if v == "**":
                b = self.expr(p)  # right associative
            else:
                b = self.expr(p + 0.01)
            a = ("bin", v, a, b)

    def primary(self):
        k, v = self.take()
        if k == "num":
            return ("num", v)
        if k == "str":
            return ("str", v[1:-1])
        if k == "dotop" and v in (".true.", ".false."):
            return ("log", v == ".true.")
        if v == "(":
            a = self.expr()
            if self.peek()[1] == ",":
                self.take()
                b = self.expr()
                self.take(")")
                return ("cplx", a, b)
            self.take(")")
            return ("paren", a)
        if k == "name":
            if self.peek()[1] == "(":
                self.take()
                args = []
                if self.peek()[1] != ")":
                    while True:
                        args.append(self.arg())
                        if self.peek()[1] == ",":
                            self.take()
                            continue
                        break
                self.take(")")
                node = ("call", v, args)
                while self.peek()[1] == "(":  # substring or chained: not used on the path
                    raise SyntaxError("chained references are not supported")
                return node
            return ("name", v)
        raise SyntaxError(f"unexpected token {v!r}")

    def arg(self):
        # keyword argument, section, or expression
        if self.peek()[0] == "name" and self.peek(1)[1] == "=" and self.peek(2)[1] != "=":
            name = self.take()[1]
            self.take("=")
            return ("kw", name, self.expr())
        lo = hi = st = None
        if self.peek()[1] != ":":
            lo = self.expr()
            if self.peek()[1] != ":":
                return lo
        self.take(":")
        if self.peek()[1] not in (",", ")", ":"):
            hi = self.expr()
        if self.peek()[1] == ":":
            self.take()
            st = self.expr()
        return ("range", lo, hi, st)


def parse_expr(s):
    p = _P(tokenize(s))
    e = p.expr()
    if p.i != len(p.t):
        raise SyntaxError(f"trailing tokens in {s!r}: {p.t[p.i:]}")
    return e


def split_top(s, sep=","):
    """Split s at top-level separators (outside parentheses and strings)."""
    out, depth, q, buf = [], 0, None, []
    for ch in s:
        if q:
            buf.append(ch)
            if ch == q:
                q = None
            continue
        if ch in "'\"":
            q = ch
        elif ch == "(":
            depth += 1
        elif ch == ")":
            depth -= 1
        elif ch == sep and depth == 0:
            out.append("".join(buf))
            buf = []
            continue
        buf.append(ch)
    out.append("".join(buf))
    return [x.strip() for x in out]


def match_paren(s, i):
    """Index of the parenthesis closing the one at s[i]."""
    depth, q = 0, None
    for j in range(i, len(s)):
        ch = s[j]
        if q:
            if ch == q:
                q = None
            continue
        if ch in "'\"":
            q = ch
        elif ch == "(":
            depth += 1
        elif ch == ")":
            depth -= 1
            if depth == 0:
                return j
    raise SyntaxError(f"unbalanced parentheses in {s!r}")


# ---------------------------------------------------------------------------
# types and storage
# type codes: 'i4', 'i8', 'r4', 'r8', 'c8', 'c16', 'l', 'ch'
_DT = {"i4": np.int32, "i8": np.int64, "r4": np.float32, "r8": np.float64, "c8": np.complex64,
       "c16": np.complex128, "l": np.bool_, "ch": object}
_SIZE = {"i4": 4, "i8": 8, "r4": 4, "r8": 8, "c8": 8, "c16": 16, "l": 4, "ch": 8}


class FArr:
    """A Fortran array: numpy array a (column-major, extents) and lower bounds.
    ext, when set, is the flat storage from the array's first element to the
    end of the COMMON block or EQUIVALENCE group that holds it (what sequence
    association may reach past the array's own end)."""
    __slots__ = ("a", "lb", "t", "ext")

    def __init__(self, a, lb, t, ext=None):
        self.a, self.lb, self.t, self.ext = a, tuple(lb), t, ext

    def flat(self):
        return self.ext if self.ext is not None else self.a.reshape(-1, order="F")

    def offset(self, idx):
        off, mult = 0, 1
        for i, l, n in zip(idx, self.lb, self.a.shape):
            off += (int(i) - l) * mult
            mult *= n
        return off


def new_storage(t, shape=None):
    if shape is None:
        return np.zeros(1, _DT[t])
    return np.zeros(shape, _DT[t], order="F")


def view_bytes(buf, off, t, shape):
    """A typed column-major view of shape into byte buffer buf at off."""
    n = int(np.prod(shape)) if shape else 1
    a = np.frombuffer(buf, dtype=_DT[t], count=n, offset=off)
    return a if not shape else a.reshape(shape, order="F")


def view_rest(buf, off, t):
    """The flat typed view of buffer buf from byte off to its end."""
    size = np.dtype(_DT[t]).itemsize
    return np.frombuffer(buf, dtype=_DT[t], count=(len(buf) - off) // size, offset=off)


class Seq:
    """An actual argument that is storage: a flat view (array name, element or
    scalar variable) passed by reference."""
    __slots__ = ("flat", "t")

    def __init__(self, flat, t):
        self.flat, self.t = flat, t


# runtime helpers used by translated code
def _idiv(a, b):
    q = abs(a) // abs(b)
    return q if (a >= 0) == (b >= 0) else -q


def _powi(x, n):
    if isinstance(x, (int, np.integer)) and not isinstance(x, bool):
        if n < 0:
            return 1 // x if abs(x) == 1 else 0
        return int(x) ** int(n)
    if n < 0:
        return 1.0 / _powi(x, -n) if not isinstance(x, np.float32) else np.float32(1) / _powi(x, -n)
    r = None
    base = x
    while n:
        if n & 1:
            r = base if r is None else r * base
        n >>= 1
        if n:
            base = base * base
    return r if r is not None else (x * 0 + 1)


def _fint(x):
    """INT(): truncation toward zero."""
    return int(x.real if isinstance(x, complex) else x)


def _nint(x):
    return int(math.floor(x + 0.5)) if x >= 0 else -int(math.floor(-x + 0.5))


def _aint(x):
    return type(x)(math.trunc(x)) if not isinstance(x, float) else float(math.trunc(x))


def _sign(a, b):
    return abs(a) if b >= 0 else -abs(a)


def _mod(a, b):
    if isinstance(a, (int, np.integer)) and isinstance(b, (int, np.integer)):
        return int(a) - _idiv(int(a), int(b)) * int(b)
    return math.fmod(a, b)


def _trip(a, b, s):
    if s == 0:
        raise ValueError("DO step 0")
    return max(0, _idiv(b - a + s, s))


def _tot(v, t):
    """Convert a Python/numpy scalar to Fortran type t."""
    if t in ("i4", "i8"):
        if isinstance(v, (complex, np.complexfloating)):
            v = v.real
        return int(v) if isinstance(v, (int, np.integer, bool, np.bool_)) else int(math.trunc(float(v)))
    if t == "r8":
        if isinstance(v, (complex, np.complexfloating)):
            return float(v.real)
        return float(v)
    if t == "r4":
        if isinstance(v, (complex, np.complexfloating)):
            v = v.real
        return np.float32(v)
    if t == "c16":
        return complex(v)
    if t == "c8":
        return np.complex64(v)
    if t == "l":
        return bool(v)
    return v


class Runtime:
    """The program: parsed units, module and COMMON storage, translated code."""

    def __init__(self):
        self.units = {}        # name -> Unit (procedures)
        self.modules = {}      # name -> Unit (modules)
        self.module_vars = {}  # module name -> dict name -> storage (cell, FArr or None)
        self.commons = {}      # block -> bytearray
        self.funcs = {}        # name -> translated python function
        self.externals = {}    # name -> python callable (stubs)
        self.files = {}        # file name -> text, for OPEN and list-directed READ
        self.units_io = {}     # unit number -> iterator over the open file's records
        self.trace = False
        # kind of CMPLX(x, y) without KIND=: default complex (REAL*4 parts),
        # as the standard says; "c16" evaluates the source as if it had
        # written KIND=8
        self.cmplx_default = "c8"

    # -- loading ---------------------------------------------------------------
    def load(self, path, includes=None):
        stmts = read_statements(path, includes)
        for u in split_units(stmts, path):
            if u.kind == "module":
                self.modules[u.name] = u
            else:
                self.units[u.name] = u

    # -- list-directed input from in-memory files --------------------------------
    def io_open(self, unit, name):
        """OPEN of a file given in self.files; OPENs of other files (the
        program's output files) are ignored like the WRITEs to them."""
        if name in self.files:
            self.units_io[int(unit)] = iter(self.files[name].splitlines())

    def io_close(self, unit):
        self.units_io.pop(int(unit), None)

    def io_read(self, unit, n):
        """The values of one list-directed READ: it starts a new record and
        reads on into the following ones until it has n values."""
        it = self.units_io.get(int(unit))
        if it is None:
            raise IOError(f"READ from unit {unit}, which has no input file open")
        vals = []
        while True:
            line = next(it).strip()
            vals += [v for v in re.split(r"[\s,]+", line) if v]
            if len(vals) >= n:
                return vals[:n]

    def provide(self, name, fn):
        """A procedure supplied in Python (a stub for MPI, or a routine whose
        source is missing from the reference tree)."""
        self.externals[name.lower()] = fn

    # -- modules -----------------------------------------------------------------
    def module(self, name):
        name = name.lower()
        if name not in self.module_vars:
            u = self.modules[name]
            scope = Scope(self, u, None)
            scope.declare_all()
            self.module_vars[name] = scope
        return self.module_vars[name]

    def var(self, module, name):
        """A module variable's storage (cell array, FArr or allocatable None)."""
        sc = self.module(module)
        return sc.storage(name.lower())

    def set_var(self, module, name, value):
        sc = self.module(module)
        sym = sc.sym[name.lower()]
        if sym.dims is not None:
            st = sc.storage(name.lower())
            if st is None or (sym.alloc and tuple(st.a.shape) != tuple(np.shape(value))):
                raise ValueError(f"{name}: allocate it first (shape {np.shape(value)})")
            st.a[...] = value
        else:
            sc.storage(name.lower())[0] = _tot(value, sym.t)

    def allocate(self, module, name, bounds):
        sc = self.module(module)
        sym = sc.sym[name.lower()]
        shape = [hi - lo + 1 for lo, hi in bounds]
        sc.values[name.lower()] = FArr(new_storage(sym.t, shape), [lo for lo, _ in bounds], sym.t)

    def common(self, block, nbytes):
        buf = self.commons.get(block)
        if buf is None or len(buf) < nbytes:
            old = buf
            buf = bytearray(max(nbytes, 8))
            if old is not None:
                buf[:len(old)] = old
            self.commons[block] = buf
        return buf

    # -- calls -------------------------------------------------------------------
    def proc(self, name):
        name = name.lower()
        if name in self.externals:
            return self.externals[name]
        f = self.funcs.get(name)
        if f is None:
            if name not in self.units:
                raise NameError(f"procedure {name} is neither in the loaded sources nor provided")
            f = translate(self, self.units[name])
            self.funcs[name] = f
        return f

    def call(self, name, *args):
        """Call a procedure with Python values: numpy arrays are passed by
        reference (as sequence storage), scalars by value."""
        conv = []
        for a in args:
            if isinstance(a, FArr):
                conv.append(Seq(a.flat(), a.t))
            elif isinstance(a, np.ndarray):
                t = {np.dtype(v): k for k, v in _DT.items()}[a.dtype]
                conv.append(Seq(a.reshape(-1, order="F") if a.ndim else a.reshape(1), t))
            elif callable(a):
                conv.append(a)
            else:
                t = ("l" if isinstance(a, (bool, np.bool_)) else "i4" if isinstance(a, (int, np.integer))
                     else "c16" if isinstance(a, complex) else "r8")
                conv.append(Seq(np.array([a], _DT[t]), t))
        return self.proc(name)(*conv)


# ---------------------------------------------------------------------------
# program units
class Unit:
    def __init__(self, kind, name, args, rtype, path):
        self.kind, self.name, self.args, self.rtype, self.path = kind, name, args, rtype, path
        self.body = []  # (label, text, lineno)


_UNIT_START = re.compile(r"^(?:(?:recursive|pure|elemental)\s+)*(?:(?P<typ>integer|real|double\s*precision|complex|logical)"
                         r"(?:\s*\*\s*\d+|\s*\([^)]*\))?\s+)?(?P<kind>subroutine|function)\s+(?P<name>\w+)\s*(?:\((?P<args>[^)]*)\))?")


def split_units(stmts, path):
    units, cur = [], None
    for lab, s, n in stmts:
        if cur is None:
            m = re.match(r"^module\s+(\w+)\s*$", s)
            if m and not s.startswith("module procedure"):
                cur = Unit("module", m.group(1), [], None, path)
                continue
            m = _UNIT_START.match(s)
            if m:
                args = [a.strip() for a in (m.group("args") or "").split(",") if a.strip()]
                cur = Unit(m.group("kind"), m.group("name"), args, m.group("typ"), path)
                continue
            m = re.match(r"^program\s+(\w+)", s)
            if m:
                cur = Unit("program", m.group(1), [], None, path)
                continue
            if s == "end" or re.match(r"^end\s*(program|subroutine|function|module)?", s):
                continue
            raise SyntaxError(f"{path}:{n}: statement outside a program unit: {s!r}")
        if re.match(r"^end\s*$", s) or re.match(r"^end\s*(subroutine|function|module|program)\b", s):
            units.append(cur)
            cur = None
            continue
        cur.body.append((lab, s, n))
    if cur is not None:
        units.append(cur)
    return units


# ---------------------------------------------------------------------------
# declarations
class Sym:
    def __init__(self, name):
        self.name = name
        self.t = None          # type code
        self.dims = None       # [(lo_expr_ast or None, hi_expr_ast or None or '*')] or None for scalars
        self.alloc = False
        self.param = None      # value of a PARAMETER
        self.param_ast = None
        self.dummy = False
        self.common = None     # (block, byte offset)
        self.equiv = None      # (group id, byte offset)
        self.save = False
        self.data = None       # list of values
        self.external = False
        self.module = None     # module scope it comes from (USE)
        self.is_proc = False


_TYPE = re.compile(r"^(?P<base>integer|real|double\s*precision|complex|logical|character)"
                   r"(?P<kind>\s*\*\s*\(?\s*\d+\s*\)?|\s*\([^)]*\))?")


def _type_code(base, kind, scope):
    base = base.replace(" ", "")
    if base == "character":
        return "ch"
    k, star = None, False
    if kind:
        kind = kind.strip()
        if kind.startswith("*"):
            k, star = int(kind[1:].strip("() ")), True
        else:
            inner = kind[1:-1]
            inner = inner.split("=")[-1].strip() if "=" in inner else inner
            k = int(scope.const(parse_expr(inner)))
    if base == "integer":
        return "i8" if k == 8 else "i4"
    if base == "real":
        return "r8" if k == 8 else "r4"
    if base == "doubleprecision":
        return "r8"
    if base == "complex":
        # COMPLEX*16 and COMPLEX(8) are double complex; COMPLEX*8, COMPLEX(4), COMPLEX single
        return "c16" if (star and k == 16) or (not star and k == 8) else "c8"
    if base == "logical":
        return "l"
    return "ch"


class Scope:
    """Symbols and storage of a unit (or a module)."""

    def __init__(self, rt, unit, caller_args):
        self.rt, self.unit = rt, unit
        self.sym = {}
        self.values = {}      # module scopes: name -> storage
        self.uses = []        # (module scope, only list or None, renames)
        self.implicit_none = False
        self.equiv_groups = []
        self.decl_done = False

    def get(self, name):
        s = self.sym.get(name)
        if s is None:
            s = self.sym[name] = Sym(name)
        return s

    def lookup(self, name):
        """The symbol of name: local, or from a USEd module."""
        if name in self.sym:
            return self, self.sym[name]
        for msc, only, ren in self.uses:
            src = ren.get(name, name)
            if only is not None and name not in only:
                continue
            r = msc.lookup(src)
            if r is not None:
                return r
        return None

    def const(self, ast):
        return Const(self).eval(ast)

    # -- declaration statements ----------------------------------------------
    def declare_all(self):
        if self.decl_done:
            return
        self.decl_done = True
        for a in self.unit.args:
            self.get(a).dummy = True
        for lab, s, n in self.unit.body:
            try:
                self.declare(s)
            except NotImplementedError:
                raise
            except Exception as e:
                raise SyntaxError(f"{self.unit.path}:{n}: {s!r}: {e}") from e
        # implicit typing
        for sym in self.sym.values():
            if sym.t is None and not sym.is_proc and sym.module is None:
                if self.implicit_none and (sym.dims is not None or sym.common or sym.dummy or sym.param_ast):
                    pass
                sym.t = "i4" if sym.name[0] in "ijklmn" else "r4"
        if self.unit.kind == "function":
            r = self.get(self.unit.name)
            if self.unit.rtype:
                r.t = _type_code(self.unit.rtype, None, self)
        # parameters
        for sym in self.sym.values():
            if sym.param_ast is not None and sym.param is None:
                sym.param = _tot(self.const(sym.param_ast), sym.t)
        if self.unit.kind == "module":
            self._module_storage()

    def declare(self, s):
        m = re.match(r"^implicit\s+none", s)
        if m:
            self.implicit_none = True
            return True
        if s.startswith("implicit"):
            raise NotImplementedError("IMPLICIT other than NONE")
        m = re.match(r"^use\s+(\w+)\s*(?:,\s*only\s*:\s*(.*))?$", s)
        if m:
            msc = self.rt.module(m.group(1))
            only, ren = None, {}
            if m.group(2) is not None:
                only = set()
                for item in split_top(m.group(2)):
                    if "=>" in item:
                        loc, src = [x.strip() for x in item.split("=>")]
                        ren[loc] = src
                        only.add(loc)
                    elif item:
                        only.add(item)
            self.uses.append((msc, only, ren))
            return True
        m = re.match(r"^parameter\s*\((.*)\)\s*$", s)
        if m:
            for item in split_top(m.group(1)):
                nm, ex = item.split("=", 1)
                sym = self.get(nm.strip())
                sym.param_ast = parse_expr(ex)
                if sym.t is None and not self.implicit_none:
                    sym.t = "i4" if sym.name[0] in "ijklmn" else "r4"
                if sym.t is not None:
                    sym.param = _tot(self.const(sym.param_ast), sym.t)
            return True
        m = re.match(r"^dimension\b\s*(?:::)?\s*(.*)$", s)
        if m:
            for ent in split_top(m.group(1).strip()):
                self._entity(ent, None, [])
            return True
        m = re.match(r"^common\s*/\s*(\w*)\s*/(.*)$", s)
        if m:
            self._common(m.group(1), m.group(2))
            return True
        m = re.match(r"^equivalence\s*(.*)$", s)
        if m:
            for grp in split_top(m.group(1)):
                grp = grp.strip()[1:-1]
                self.equiv_groups.append([parse_expr(x) for x in split_top(grp)])
            return True
        m = re.match(r"^external\s*(?:::)?\s*(.*)$", s)
        if m:
            for nm in split_top(m.group(1)):
                sym = self.get(nm)
                sym.external = sym.is_proc = True
            return True
        if re.match(r"^intrinsic\b", s):
            return True
        m = re.match(r"^save\s*(.*)$", s)
        if m:
            items = [x for x in split_top(m.group(1).replace("::", "")) if x]
            if not items:
                self._save_all = True
            for nm in items:
                if not nm.startswith("/"):
                    self.get(nm).save = True
            return True
        m = re.match(r"^data\s+(.*)$", s)
        if m:
            self._data(m.group(1))
            return True
        m = _TYPE.match(s)
        if m and not re.match(r"^(real|integer|complex|logical)\s*\w*\s*\(.*\)\s*=", s) \
                and not re.match(r"^(integer|real|double\s*precision|complex|logical)(\s*\*\s*\d+|\s*\([^)]*\))?\s*function\b", s):
            rest = s[m.end():]
            attrs = []
            if "::" in rest:
                a, rest = rest.split("::", 1)
                attrs = [x.strip() for x in split_top(a) if x.strip()]
            t = _type_code(m.group("base"), m.group("kind"), self)
            for ent in split_top(rest.strip()):
                if ent:
                    self._entity(ent, t, attrs)
            return True
        return False

    def _dims(self, text):
        out = []
        for d in split_top(text):
            if d == "*":
                out.append((None, "*"))
            elif d == ":":
                out.append((None, None))
            elif ":" in d:
                lo, hi = d.split(":", 1)
                out.append((parse_expr(lo), "*" if hi.strip() == "*" else (parse_expr(hi) if hi.strip() else None)))
            else:
                out.append((("num", "1"), parse_expr(d)))
        return out

    def _entity(self, ent, t, attrs):
        init = None
        if "=" in ent and "=>" not in ent:
            ent, init = ent.split("=", 1)
            ent = ent.strip()
        m = re.match(r"^(\w+)\s*(?:\*\s*(\d+))?\s*(\((.*)\))?\s*(?:\*\s*\d+)?$", ent)
        if not m:
            raise SyntaxError(f"entity {ent!r}")
        sym = self.get(m.group(1))
        if t is not None:
            sym.t = t
        if m.group(3):
            sym.dims = self._dims(m.group(4))
        for a in attrs:
            if a == "parameter":
                sym.param_ast = parse_expr(init)
                init = None
            elif a == "allocatable":
                sym.alloc = True
            elif a.startswith("dimension"):
                sym.dims = self._dims(a[a.index("(") + 1:a.rindex(")")])
            elif a == "save":
                sym.save = True
            elif a == "external":
                sym.external = sym.is_proc = True
            # intent, target, optional: no effect here
        if init is not None and sym.param_ast is None:
            sym.data = [parse_expr(init)]
            sym.save = True
        if sym.param_ast is not None and sym.t is not None:
            sym.param = _tot(self.const(sym.param_ast), sym.t)

    def _common(self, block, text):
        # possibly several blocks: /a/ x, y /b/ z
        parts = re.split(r"/\s*(\w*)\s*/", "/" + block + "/" + text)
        names = parts[1::2]
        lists = parts[2::2]
        for blk, lst in zip(names, lists):
            items = [x for x in split_top(lst.strip().rstrip(",")) if x]
            self.__dict__.setdefault("_commons", []).append((blk or "_blank_", items))
            for it in items:
                m = re.match(r"^(\w+)\s*(\((.*)\))?$", it)
                sym = self.get(m.group(1))
                if m.group(2):
                    sym.dims = self._dims(m.group(3))
                sym.common = (blk or "_blank_", None)

    def _data(self, text):
        # name-list /values/ [, name-list /values/ ...]
        for m in re.finditer(r"([^/]+)/([^/]*)/\s*,?", text):
            names = [x for x in split_top(m.group(1).strip().rstrip(",")) if x]
            vals = []
            for v in split_top(m.group(2)):
                if "*" in v and re.match(r"^\d+\s*\*", v):
                    k, w = v.split("*", 1)
                    vals += [parse_expr(w)] * int(k)
                else:
                    vals.append(parse_expr(v))
            for nm in names:
                sym = self.get(nm.strip())
                sym.data = vals
                sym.save = True

    # -- storage layout (COMMON, EQUIVALENCE, modules) ------------------------
    def shape_of(self, sym, evaluator):
        if sym.dims is None:
            return None
        shape, lbs = [], []
        for lo, hi in sym.dims:
            l = 1 if lo is None else int(evaluator(lo))
            if hi == "*" or hi is None:
                return None, None
            h = int(evaluator(hi))
            shape.append(max(0, h - l + 1))
            lbs.append(l)
        return shape, lbs

    def static_layout(self):
        """Byte layout of COMMON blocks and EQUIVALENCE groups of this unit:
        {name: (buffer key, byte offset)} and the buffers' sizes."""
        lay, sizes = {}, {}
        cev = lambda e: self.const(e)
        for blk, items in getattr(self, "_commons", []):
            off = 0
            for it in items:
                nm = re.match(r"^(\w+)", it).group(1)
                sym = self.sym[nm]
                shp = self.shape_of(sym, cev)
                n = int(np.prod(shp[0])) if shp else 1
                lay[nm] = (("common", blk), off)
                off += n * _SIZE[sym.t]
            key = ("common", blk)
            sizes[key] = max(sizes.get(key, 0), off)
        for gi, grp in enumerate(self.equiv_groups):
            # the first member anchors the group (its own storage or its common)
            offs = {}
            for e in grp:
                nm, idx = (e[1], []) if e[0] == "name" else (e[1], e[2])
                sym = self.sym[nm]
                shp = self.shape_of(sym, cev)
                eoff = 0
                if idx:
                    mult = 1
                    for (ix, l, n) in zip(idx, shp[1], shp[0]):
                        eoff += (int(self.const(ix)) - l) * mult
                        mult *= n
                offs[nm] = eoff * _SIZE[sym.t]
            anchor = next((nm for nm in offs if nm in lay), None)
            if anchor is not None:
                key, aoff = lay[anchor]
                base = aoff + offs[anchor]
            else:
                key, base = ("equiv", self.unit.name, gi), 0
                # place every member so that none starts before byte 0
                base = max(offs.values())
            for nm, o in offs.items():
                if nm in lay and nm != anchor:
                    continue
                lay[nm] = (key, base - o)
                sym = self.sym[nm]
                shp = self.shape_of(sym, cev)
                n = int(np.prod(shp[0])) if shp else 1
                sizes[key] = max(sizes.get(key, 0), base - o + n * _SIZE[sym.t])
        return lay, sizes

    def _module_storage(self):
        lay, sizes = self.static_layout()
        bufs = {}
        for key, nbytes in sizes.items():
            bufs[key] = self.rt.common(key[1], nbytes) if key[0] == "common" else bytearray(nbytes)
        for nm, sym in self.sym.items():
            if sym.param is not None or sym.is_proc or sym.module is not None:
                continue
            if sym.t is None:
                continue
            if sym.alloc:
                self.values[nm] = None
                continue
            shp = self.shape_of(sym, lambda e: self.const(e))
            if nm in lay:
                key, off = lay[nm]
                st = view_bytes(bufs[key], off, sym.t, shp[0] if shp else None)
                self.values[nm] = FArr(st, shp[1], sym.t, view_rest(bufs[key], off, sym.t)) if shp else st
            else:
                self.values[nm] = FArr(new_storage(sym.t, shp[0]), shp[1], sym.t) if shp else new_storage(sym.t)
            if sym.data:
                _apply_data(self, sym, self.values[nm])

    def storage(self, name):
        return self.values.get(name)


def _apply_data(scope, sym, st):
    vals = [_tot(scope.const(v), sym.t) for v in sym.data]
    if isinstance(st, FArr):
        f = st.flat()
        f[:len(vals)] = vals
    else:
        st[0] = vals[0]


class Const:
    """Evaluation of constant expressions (PARAMETER values, bounds of
    module arrays)."""

    def __init__(self, scope):
        self.scope = scope

    def eval(self, e):
        k = e[0]
        if k == "num":
            return _num_value(e[1])[0]
        if k == "paren":
            return self.eval(e[1])
        if k == "un":
            v = self.eval(e[2])
            return -v if e[1] == "-" else v if e[1] == "+" else (not v)
        if k == "bin":
            a, b = self.eval(e[2]), self.eval(e[3])
            op = e[1]
            if op == "+": return a + b
            if op == "-": return a - b
            if op == "*": return a * b
            if op == "/": return _idiv(a, b) if isinstance(a, int) and isinstance(b, int) else a / b
            if op == "**": return _powi(a, b) if isinstance(b, int) else a ** b
            raise ValueError(op)
        if k == "name":
            r = self.scope.lookup(e[1])
            if r is None or r[1].param_ast is None:
                raise ValueError(f"{e[1]} is not a constant")
            sc, sym = r
            if sym.param is None:
                sym.param = _tot(sc.const(sym.param_ast), sym.t or ("i4" if sym.name[0] in "ijklmn" else "r4"))
            return sym.param
        if k == "call":
            f, args = e[1], [self.eval(a) for a in e[2] if a[0] != "kw"]
            if f == "ceiling": return int(math.ceil(args[0]))
            if f == "floor": return int(math.floor(args[0]))
            if f == "real": return float(np.float32(args[0]))
            if f in ("dble", "float"): return float(args[0])
            if f == "int": return int(args[0])
            if f == "max": return max(args)
            if f == "min": return min(args)
            if f == "mod": return _mod(args[0], args[1])
            if f == "kind": return 8 if isinstance(args[0], float) else 4
            if f == "selected_real_kind": return 8
            if f == "abs": return abs(args[0])
            raise ValueError(f"intrinsic {f} in a constant")
        if k == "cplx":
            return complex(self.eval(e[1]), self.eval(e[2]))
        if k == "log":
            return e[1]
        raise ValueError(f"constant {e}")


def _num_value(text):
    """(value, type code) of a numeric literal."""
    kind = None
    if "_" in text:
        text, kind = text.split("_", 1)
    if re.match(r"^\d+$", text):
        return int(text), "i8" if kind in ("8", "i8") else "i4"
    dbl = "d" in text
    v = float(text.replace("d", "e"))
    if dbl or kind in ("8", "r8", "dp"):
        return v, "r8"
    return float(np.float32(v)), "r4"


# ---------------------------------------------------------------------------
# translation of a procedure into Python
_INTRINSIC_TYPE = {"abs": None, "iabs": "i4", "dabs": "r8", "sqrt": None, "dsqrt": "r8", "exp": None, "dexp": "r8",
                   "log": None, "dlog": "r8", "sin": None, "cos": None, "tan": None, "tanh": None, "dtanh": "r8",
                   "atan": None, "atan2": None, "datan": "r8", "dsin": "r8", "dcos": "r8"}


class Translator:
    def __init__(self, rt, unit):
        self.rt, self.unit = rt, unit
        self.sc = Scope(rt, unit, None)
        self.sc.declare_all()
        self.lines = []
        self.tmp = 0
        self.regs = set()      # scalar locals kept in Python variables
        self.goto_labels = set()
        self.ctx = {}          # objects bound into the function's globals
        self.do_stack = []
        self.modrefs = {}

    # -- names -------------------------------------------------------------------
    def emit(self, s, ind):
        self.lines.append("    " * ind + s)

    def newtmp(self):
        self.tmp += 1
        return f"_t{self.tmp}"

    def bind(self, obj, hint="o"):
        k = f"_{hint}{len(self.ctx)}"
        self.ctx[k] = obj
        return k

    def resolve(self, name):
        """(kind, symbol, python ref): kind in local, dummy, module, param, proc."""
        if name in self.sc.sym:
            sym = self.sc.sym[name]
            if sym.param is not None or sym.param_ast is not None:
                if sym.param is None:
                    sym.param = _tot(self.sc.const(sym.param_ast), sym.t)
                return "param", sym, repr(sym.param)
            if sym.is_proc and not sym.dummy:
                return "proc", sym, name
            if sym.dummy:
                return "dummy", sym, f"v_{name}"
            return "local", sym, f"v_{name}"
        r = self.sc.lookup(name)
        if r is not None:
            msc, sym = r
            if sym.param is not None or sym.param_ast is not None:
                if sym.param is None:
                    sym.param = _tot(msc.const(sym.param_ast), sym.t)
                return "param", sym, repr(sym.param)
            key = self.modrefs.get(id(msc))
            if key is None:
                key = self.modrefs[id(msc)] = self.bind(msc, "m")
            return "module", sym, f"{key}.values[{sym.name!r}]"
        return None, None, None

    # -- expressions -------------------------------------------------------------
    def ex(self, e):
        """(python code, type code, is_array) of an expression."""
        k = e[0]
        if k == "num":
            v, t = _num_value(e[1])
            if t == "r4":
                return f"_f32({v!r})", "r4", False
            return repr(v), t, False
        if k == "log":
            return repr(e[1]), "l", False
        if k == "str":
            return repr(e[1]), "ch", False
        if k == "paren":
            c, t, a = self.ex(e[1])
            return f"({c})", t, a
        if k == "cplx":
            (cr, tr, _), (ci, ti, _) = self.ex(e[1]), self.ex(e[2])
            t = "c16" if "r8" in (tr, ti) else "c8"
            conv = "complex" if t == "c16" else "_c64"
            return f"{conv}({cr}, {ci})", t, False
        if k == "name":
            return self.ex_name(e[1])
        if k == "call":
            return self.ex_call(e)
        if k == "un":
            c, t, a = self.ex(e[2])
            if e[1] == ".not.":
                return f"(not {c})" if not a else f"(~{c})", "l", a
            return f"({e[1]}{c})", t, a
        if k == "bin":
            return self.ex_bin(e)
        raise NotImplementedError(f"expression {e}")

    def ex_name(self, name):
        kind, sym, ref = self.resolve(name)
        if kind is None:
            raise NameError(f"{self.unit.name}: unknown name {name}")
        if kind == "param":
            t = sym.t
            if t == "r4":
                return f"_f32({sym.param!r})", t, False
            return ref, t, False
        if kind == "proc":
            raise NotImplementedError(f"procedure name {name} used as a value")
        if sym.dims is not None:
            return f"{ref}.a", sym.t, True
        if name in self.regs:
            return f"r_{name}", sym.t, False
        return f"{ref}[0]", sym.t, False

    def conv(self, code, frm, to):
        if frm == to or to is None:
            return code
        if to in ("i4", "i8"):
            if frm in ("i4", "i8"):
                return code
            return f"_fint({code})"
        if to == "r8":
            if frm in ("c8", "c16"):
                return f"({code}).real"
            return f"float({code})"
        if to == "r4":
            return f"_f32({code})"
        if to == "c16":
            return f"complex({code})"
        if to == "c8":
            return f"_c64({code})"
        if to == "l":
            return code
        return code

    _RANK = {"i4": 1, "i8": 2, "r4": 3, "r8": 4, "c8": 5, "c16": 6}

    def common_type(self, ta, tb):
        if ta == tb:
            return ta
        if {ta, tb} <= {"i4", "i8"}:
            return "i8"
        if "c16" in (ta, tb) or ({ta, tb} & {"c8"} and {ta, tb} & {"r8"}):
            return "c16"
        if "c8" in (ta, tb):
            return "c8"
        if "r8" in (ta, tb):
            return "r8"
        return "r4"

    def ex_bin(self, e):
        op = e[1]
        ca, ta, aa = self.ex(e[2])
        cb, tb, ab = self.ex(e[3])
        arr = aa or ab
        rel = {".eq.": "==", ".ne.": "!=", ".lt.": "<", ".le.": "<=", ".gt.": ">", ".ge.": ">=",
               "==": "==", "/=": "!=", "<": "<", "<=": "<=", ">": ">", ">=": ">="}
        if op in rel:
            t = self.common_type(ta, tb) if ta != "l" else "l"
            return f"({self.conv(ca, ta, t)} {rel[op]} {self.conv(cb, tb, t)})", "l", arr
        if op in (".and.", ".or."):
            if arr:
                return f"({ca} {'&' if op == '.and.' else '|'} {cb})", "l", True
            return f"({ca} {op[1:-1]} {cb})", "l", False
        if op in (".eqv.", ".neqv."):
            return f"({ca} {'==' if op == '.eqv.' else '!='} {cb})", "l", arr
        if op == "**":
            if tb in ("i4", "i8"):
                if arr:
                    return f"({ca} ** {cb})", ta, True
                return f"_powi({ca}, {cb})", ta, False
            t = self.common_type(ta, tb)
            return f"({self.conv(ca, ta, t)} ** {self.conv(cb, tb, t)})", t, arr
        t = self.common_type(ta, tb)
        a, b = self.conv(ca, ta, t), self.conv(cb, tb, t)
        if op == "/" and t in ("i4", "i8"):
            if arr:
                return f"_idiv_arr({a}, {b})", t, True
            return f"_idiv({a}, {b})", t, False
        if op == "//":
            return f"({a} + {b})", "ch", False
        return f"({a} {op} {b})", t, arr

    def index_code(self, ref, sym, args):
        """numpy index of array ref by Fortran subscripts (elements or sections)."""
        parts, arr = [], False
        for i, a in enumerate(args):
            lb = f"{ref}.lb[{i}]"
            if a[0] == "range":
                lo = "" if a[1] is None else f"{self.int_ex(a[1])}-{lb}"
                hi = "" if a[2] is None else f"{self.int_ex(a[2])}-{lb}+1"
                st = "" if a[3] is None else f":{self.int_ex(a[3])}"
                parts.append(f"{lo}:{hi}{st}")
                arr = True
            else:
                c, t, isarr = self.ex(a)
                if isarr:
                    raise NotImplementedError("vector subscripts")
                parts.append(f"{self.conv(c, t, 'i8')}-{lb}")
        return ", ".join(parts), arr

    def int_ex(self, e):
        c, t, a = self.ex(e)
        return self.conv(c, t, "i8")

    def ex_call(self, e):
        name, args = e[1], e[2]
        kind, sym, ref = self.resolve(name)
        if kind in ("local", "dummy", "module") and sym.dims is not None:
            idx, arr = self.index_code(ref, sym, args)
            return f"{ref}.a[{idx}]", sym.t, arr
        if kind == "proc" or (kind is None and (name in self.rt.units or name in self.rt.externals)):
            # a user function
            call = self.call_code(name, args, kind == "dummy")
            t = self.function_type(name)
            return call, t, False
        if kind == "dummy" and sym.is_proc:
            return self.call_code(name, args, True), sym.t or "r8", False
        return self.intrinsic(name, args)

    def function_type(self, name):
        u = self.rt.units.get(name)
        if u is not None and u.rtype:
            return _type_code(u.rtype, None, self.sc)
        sym = self.sc.sym.get(name)
        if sym is not None and sym.t:
            return sym.t
        return "i4" if name[0] in "ijklmn" else "r4"

    def intrinsic(self, name, args):
        ev = [self.ex(a) for a in args if a[0] != "kw"]
        kw = {a[1]: self.ex(a[2]) for a in args if a[0] == "kw"}
        arr = any(x[2] for x in ev)
        npfx = "np." if arr else ""
        def one(t=None):
            c, tt, _ = ev[0]
            return self.conv(c, tt, t) if t else c
        if name in ("abs", "iabs", "dabs", "cabs"):
            c, t, _ = ev[0]
            if t in ("c8", "c16"):
                return f"abs({c})", "r8" if t == "c16" else "r4", arr
            return (f"np.abs({c})" if arr else f"abs({c})"), t, arr
        if name in ("sqrt", "dsqrt", "exp", "dexp", "log", "dlog", "sin", "dsin", "cos", "dcos", "tan", "tanh",
                    "dtanh", "atan", "datan"):
            c, t, _ = ev[0]
            fn = name[1:] if name.startswith("d") and name not in ("dlog",) else ("log" if name == "dlog" else name)
            if name == "dlog":
                fn = "log"
            if t in ("c8", "c16"):
                return f"_cmath.{fn}({c})", t, arr
            if t == "r4":
                return f"_f32(np.{fn}(np.float32({c})))", "r4", arr
            tt = "r8" if t in ("i4", "i8", "r8") else t
            return (f"np.{fn}({self.conv(c, t, tt)})" if arr else f"_math.{fn}({self.conv(c, t, tt)})"), tt, arr
        if name in ("atan2", "datan2"):
            (a, ta, _), (b, tb, _) = ev[0], ev[1]
            return f"_math.atan2({self.conv(a, ta, 'r8')}, {self.conv(b, tb, 'r8')})", "r8", False
        if name in ("max", "min", "amax1", "amin1", "dmax1", "dmin1", "max0", "min0"):
            t = ev[0][1]
            for _, tt, _ in ev[1:]:
                t = self.common_type(t, tt)
            vals = ", ".join(self.conv(c, tt, t) for c, tt, _ in ev)
            fn = "max" if "max" in name else "min"
            if arr:
                red = "np.maximum" if fn == "max" else "np.minimum"
                code = self.conv(ev[0][0], ev[0][1], t)
                for c, tt, _ in ev[1:]:
                    code = f"{red}({code}, {self.conv(c, tt, t)})"
                return code, t, True
            return f"{fn}({vals})", t, False
        if name in ("mod", "dmod"):
            (a, ta, _), (b, tb, _) = ev[0], ev[1]
            t = self.common_type(ta, tb)
            return f"_mod({self.conv(a, ta, t)}, {self.conv(b, tb, t)})", t, False
        if name in ("sign", "dsign", "isign"):
            (a, ta, _), (b, tb, _) = ev[0], ev[1]
            return f"_sign({a}, {b})", ta, False
        if name in ("float", "real", "sngl", "dble", "dfloat"):
            c, t, _ = ev[0]
            to = "r8" if name in ("dble", "dfloat") else "r4"
            if "kind" in kw or len(ev) > 1:
                kc = kw["kind"][0] if "kind" in kw else ev[1][0]
                to = "r8" if eval(kc, {"_f32": np.float32}) == 8 else "r4"
            if t in ("c8", "c16"):
                return (f"({c}).real" if to == "r8" else f"_f32(({c}).real)"), to, arr
            if arr:
                return f"({c}).astype({'np.float64' if to == 'r8' else 'np.float32'})", to, True
            return self.conv(c, t, to), to, False
        if name in ("int", "idint", "ifix"):
            c, t, _ = ev[0]
            return self.conv(c, t, "i4"), "i4", arr
        if name in ("nint", "idnint"):
            return f"_nint({ev[0][0]})", "i4", False
        if name in ("aint", "dint"):
            c, t, _ = ev[0]
            return f"_aint({c})", t, False
        if name in ("ceiling",):
            return f"_math.ceil({ev[0][0]})", "i4", False
        if name in ("floor",):
            return f"_math.floor({ev[0][0]})", "i4", False
        if name in ("cmplx", "dcmplx"):
            (a, ta, _) = ev[0]
            b, tb = (ev[1][0], ev[1][1]) if len(ev) > 1 else ("0.0", "r8")
            to = "c16" if name == "dcmplx" else self.rt.cmplx_default
            if "kind" in kw:
                to = "c16" if eval(kw["kind"][0]) == 8 else "c8"
            if to == "c16":
                return f"complex({self.conv(a, ta, 'r8')}, {self.conv(b, tb, 'r8')})", "c16", False
            return f"_c64(complex(float(_f32({self.conv(a, ta, 'r8')})), float(_f32({self.conv(b, tb, 'r8')}))))", \
                "c8", False
        if name in ("aimag", "dimag", "imag"):
            c, t, _ = ev[0]
            return (f"({c}).imag" if not arr else f"np.imag({c})"), ("r8" if t == "c16" else "r4"), arr
        if name in ("conjg", "dconjg"):
            c, t, _ = ev[0]
            return (f"({c}).conjugate()"), t, arr
        if name == "sum":
            c, t, _ = ev[0]
            return f"np.sum({c})", t, False
        if name == "maxval":
            return f"np.max({ev[0][0]})", ev[0][1], False
        if name in ("ieee_is_nan", "isnan"):
            c, t, _ = ev[0]
            return (f"np.isnan({c})" if arr else f"_math.isnan({c})"), "l", arr
        if name == "minval":
            return f"np.min({ev[0][0]})", ev[0][1], False
        if name == "allocated":
            return f"({ev[0][0].replace('.a', '')} is not None)", "l", False
        if name == "size":
            return f"{ev[0][0]}.size", "i4", False
        if name == "epsilon":
            return ("float(np.finfo(np.float64).eps)", "r8", False)
        raise NotImplementedError(f"{self.unit.name}: intrinsic or unknown function {name}")

    # -- calls ---------------------------------------------------------------------
    def actual(self, a):
        """Python code of an actual argument (by reference where possible)."""
        if a[0] == "name":
            kind, sym, ref = self.resolve(a[1])
            if kind in ("local", "dummy", "module"):
                if sym.is_proc:
                    return ref if kind == "dummy" else f"_rt.proc({a[1]!r})"
                if sym.dims is not None:
                    return f"_Seq({ref}.flat(), {sym.t!r})"
                if a[1] in self.regs:
                    raise RuntimeError(f"register {a[1]} passed by reference")
                return f"_Seq({ref}, {sym.t!r})"
            if kind == "proc" or (kind is None and (a[1] in self.rt.units or a[1] in self.rt.externals)):
                return f"_rt.proc({a[1]!r})"
        if a[0] == "call":
            kind, sym, ref = self.resolve(a[1])
            if kind in ("local", "dummy", "module") and sym.dims is not None and \
                    all(x[0] != "range" for x in a[2]):
                idx = ", ".join(self.int_ex(x) for x in a[2])
                return f"_elem({ref}, ({idx},))"
            if kind in ("local", "dummy", "module") and sym.dims is not None:
                idx, _ = self.index_code(ref, sym, a[2])
                return f"_section({ref}.a[{idx}], {sym.t!r})"
        c, t, arr = self.ex(a)
        if arr:
            return f"_Seq(np.array({c}).reshape(-1, order='F'), {t!r})"
        return f"_Seq(np.array([{c}], _DT[{t!r}]), {t!r})"

    def call_code(self, name, args, dummy_proc=False):
        acts = ", ".join(self.actual(a) for a in args)
        if dummy_proc:
            return f"v_{name}({acts})"
        return f"_rt.proc({name!r})({acts})"

    # -- statements ------------------------------------------------------------------
    def translate(self):
        u = self.unit
        body = [(lab, s, n) for lab, s, n in u.body if not self.is_decl(s)]
        self.find_regs(body)
        for lab, s, n in body:
            for m in re.finditer(r"go\s*to\s*(\d+)", s):
                self.goto_labels.add(int(m.group(1)))
        args = ", ".join(f"a_{a}" for a in u.args)
        self.emit(f"def f_{u.name}({args}):", 0)
        self.prologue(1)
        tree = self.structure(body)
        self.block(tree, 1, top=True)
        self.emit(self.return_code(), 1)
        src = "\n".join(self.lines)
        g = dict(_GLOBALS)
        g.update(self.ctx)
        g["_rt"] = self.rt
        try:
            exec(compile(src, f"<fortran {u.name}>", "exec"), g)
        except SyntaxError as e:
            raise SyntaxError(f"translation of {u.name} failed: {e}\n{src}") from e
        f = g[f"f_{u.name}"]
        f.__source__ = src
        return f

    def return_code(self):
        if self.unit.kind == "function":
            return f"return {self.ex_name(self.unit.name)[0]}"
        return "return None"

    def is_decl(self, s):
        if re.match(r"^(implicit|use|parameter|dimension|common|equivalence|external|intrinsic|save|data)\b", s):
            return True
        if re.match(r"^(integer|real|double\s*precision|complex|logical|character)\b", s) and \
                not re.match(r"^(integer|real|double\s*precision|complex|logical|character)\w*\s*\(.*\)\s*=", s):
            return True
        if re.match(r"^format\b", s) or re.match(r"^\d+\s+format", s):
            return True
        return False

    def find_regs(self, body):
        """Local scalars never passed by reference, not in storage
        association, not saved: Python variables."""
        passed = set()

        def walk(e):
            if not isinstance(e, tuple):
                return
            if e[0] == "call":
                kind, sym, _ = self.resolve(e[1]) if e[1] in self.sc.sym or self.sc.lookup(e[1]) else (None, None, None)
                is_array = sym is not None and sym.dims is not None
                for a in e[2]:
                    if not is_array and isinstance(a, tuple) and a[0] == "name":
                        passed.add(a[1])
                    walk(a)
                return
            for x in e[1:]:
                if isinstance(x, tuple):
                    walk(x)
                elif isinstance(x, list):
                    for y in x:
                        walk(y)

        for lab, s, n in body:
            for m in re.finditer(r"\bcall\s+(\w+)\s*(\(.*\))?\s*$", s):
                if m.group(2):
                    for a in _P(tokenize(m.group(2))).primary_args():
                        if isinstance(a, tuple) and a[0] == "name":
                            passed.add(a[1])
                        walk(a)
            i = _assign_split(s)
            if i is not None:
                try:
                    walk(parse_expr(s[i + 1:]))
                except SyntaxError:
                    pass
        for nm, sym in self.sc.sym.items():
            if sym.dims is None and not sym.dummy and sym.common is None and not sym.save and \
                    sym.param_ast is None and not sym.is_proc and sym.t in ("i4", "i8", "r8", "c16", "l") and \
                    nm not in passed and nm != self.unit.name and not self.in_equiv(nm):
                self.regs.add(nm)

    def in_equiv(self, nm):
        for grp in self.sc.equiv_groups:
            for e in grp:
                if e[1] == nm:
                    return True
        return False

    def prologue(self, ind):
        sc, u = self.sc, self.unit
        lay, sizes = sc.static_layout()
        static = self.rt.__dict__.setdefault("_static", {})
        bufs = {}
        for key, nbytes in sizes.items():
            if key[0] == "common":
                bufs[key] = self.bind(self.rt.common(key[1], nbytes), "cb")
            else:
                skey = (u.name, key)
                if skey not in static:
                    static[skey] = bytearray(nbytes)
                bufs[key] = self.bind(static[skey], "eq")
        # scalar dummies first (bounds of dummy arrays may use them)
        for a in u.args:
            sym = sc.sym[a]
            if sym.is_proc or (sym.t is None and sym.external):
                self.emit(f"v_{a} = a_{a}", ind)
            elif sym.dims is None:
                self.emit(f"v_{a} = _scalar_arg(a_{a}, {sym.t!r})", ind)
        later = []  # dummy arrays, then automatic local arrays: their bounds may use anything above
        for nm, sym in sc.sym.items():
            if sym.param_ast is not None or sym.is_proc or sym.module is not None:
                continue
            if sym.dummy and sym.dims is None:
                continue
            if sym.t is None:
                continue
            if nm in self.regs:
                init = {"i4": "0", "i8": "0", "r8": "0.0", "c16": "0j", "l": "False"}[sym.t]
                self.emit(f"r_{nm} = {init}", ind)
                continue
            if sym.dims is None and nm == u.name and u.kind == "function":
                self.emit(f"v_{nm} = np.zeros(1, _DT[{sym.t!r}])", ind)
                continue
            dims = sym.dims
            if sym.dummy:
                later.append((0, nm, sym))
                continue
            if nm in lay:
                key, off = lay[nm]
                if dims is None:
                    self.emit(f"v_{nm} = _view({bufs[key]}, {off}, {sym.t!r}, None)", ind)
                else:
                    shape, lbs = sc.shape_of(sym, lambda e: sc.const(e))
                    self.emit(f"v_{nm} = _FArr(_view({bufs[key]}, {off}, {sym.t!r}, {tuple(shape)}), "
                              f"{tuple(lbs)}, {sym.t!r}, _view_rest({bufs[key]}, {off}, {sym.t!r}))", ind)
                continue
            if sym.save:
                skey = (u.name, nm)
                if skey not in static:
                    if dims is None:
                        st = new_storage(sym.t)
                    else:
                        shape, lbs = sc.shape_of(sym, lambda e: sc.const(e))
                        st = FArr(new_storage(sym.t, shape), lbs, sym.t)
                    if sym.data:
                        _apply_data(sc, sym, st)
                    static[skey] = st
                self.emit(f"v_{nm} = {self.bind(static[skey], 's')}", ind)
                continue
            if dims is None:
                self.emit(f"v_{nm} = np.zeros(1, _DT[{sym.t!r}])", ind)
            elif sym.alloc:
                self.emit(f"v_{nm} = None", ind)
            else:
                later.append((1, nm, sym))
        for k, nm, sym in sorted(later, key=lambda x: x[0]):
            lbs, exts = [], []
            for lo, hi in sym.dims:
                l = "1" if lo is None else self.int_ex(lo)
                lbs.append(l)
                if k == 0:
                    exts.append("None" if hi in ("*", None) else f"({self.int_ex(hi)})-({l})+1")
                else:
                    exts.append(f"({self.int_ex(hi)})-({l})+1")
            if k == 0:
                self.emit(f"v_{nm} = _array_arg(a_{nm}, {sym.t!r}, [{', '.join(lbs)}], [{', '.join(exts)}])", ind)
            else:
                self.emit(f"v_{nm} = _FArr(np.zeros(({', '.join(exts)},), _DT[{sym.t!r}], order='F'), "
                          f"({', '.join(lbs)},), {sym.t!r})", ind)

    # structure: a list of nodes: ('s', lab, text, n) | ('if', lab, [(cond, body)], else_body, n) |
    # ('do', lab, var, range, body, endlabel, n) | ('while', lab, cond, body, n)
    def structure(self, body):
        pos = 0
        ended = []  # labels of labeled DOs closed by the statement just consumed

        def parse_block(end_pred, end_label=None):
            nonlocal pos
            out = []
            while pos < len(body):
                if end_label is not None and ended and ended[-1] == end_label:
                    return out  # an inner DO shared our terminal statement
                lab, s, n = body[pos]
                if end_pred(lab, s):
                    return out
                pos += 1
                if re.match(r"^if\s*\(", s) and _if_then(s):
                    i = s.index("(")
                    cond = s[i + 1:match_paren(s, i)]
                    arms, els = [], None
                    while True:
                        blk = parse_block(lambda l, t: re.match(r"^(else\s*if\b|else$|end\s*if$)", t))
                        arms.append((cond, blk))
                        lab2, s2, n2 = body[pos]
                        pos += 1
                        if re.match(r"^else\s*if", s2):
                            i = s2.index("(")
                            cond = s2[i + 1:match_paren(s2, i)]
                            continue
                        if s2 == "else":
                            els = parse_block(lambda l, t: re.match(r"^end\s*if$", t))
                            pos += 1
                        break
                    out.append(("if", lab, arms, els, n))
                    continue
                m = re.match(r"^do\s+(\d+)\s*,?\s*(\w+)\s*=\s*(.*)$", s)
                if m:
                    endl = int(m.group(1))
                    var, rng = m.group(2), split_top(m.group(3))
                    blk = parse_block(lambda l, t: l == endl, endl)
                    if ended and ended[-1] == endl:
                        out.append(("do", lab, var, rng, blk, endl, n))
                        continue
                    lab2, s2, n2 = body[pos]
                    pos += 1
                    if not re.match(r"^continue$", s2) and not re.match(r"^end\s*do$", s2):
                        blk.append(("s", None, s2, n2))  # a labeled action statement ends the loop
                    ended.append(endl)
                    out.append(("do", lab, var, rng, blk, endl, n))
                    continue
                if ended:
                    ended.clear()
                m = re.match(r"^select\s*case\s*\((.*)\)$", s)
                if m:
                    arms = []
                    stop = lambda l, t: re.match(r"^(case\b|end\s*select$)", t)
                    if parse_block(stop):
                        raise NotImplementedError("statements between SELECT CASE and its first CASE")
                    while True:
                        lab2, s2, n2 = body[pos]
                        pos += 1
                        if re.match(r"^end\s*select$", s2):
                            break
                        mc = re.match(r"^case\s*(default$|\((.*)\)$)", s2)
                        if not mc:
                            raise NotImplementedError(f"statement {s2!r}")
                        sel = None if mc.group(1) == "default" else split_top(mc.group(2))
                        arms.append((sel, parse_block(stop)))
                    out.append(("select", lab, m.group(1), arms, n))
                    continue
                m = re.match(r"^do\s+while\s*\((.*)\)$", s)
                if m:
                    blk = parse_block(lambda l, t: re.match(r"^end\s*do$", t))
                    pos += 1
                    out.append(("while", lab, m.group(1), blk, n))
                    continue
                m = re.match(r"^do\s+(\w+)\s*=\s*(.*)$", s)
                if m:
                    var, rng = m.group(1), split_top(m.group(2))
                    blk = parse_block(lambda l, t: re.match(r"^end\s*do$", t))
                    lab2, s2, n2 = body[pos]
                    pos += 1
                    out.append(("do", lab, var, rng, blk, lab2, n))
                    continue
                out.append(("s", lab, s, n))
            return out

        return parse_block(lambda l, t: False)

    def block(self, nodes, ind, top=False):
        if top and self.goto_labels:
            # top-level dispatcher: blocks from each goto target on
            cuts = [i for i, nd in enumerate(nodes) if nd[1] in self.goto_labels]
            starts = sorted(set([0] + cuts))
            self.emit("_pc = 0", ind)
            self.emit("while True:", ind)
            self.emit("try:", ind + 1)
            for bi, st in enumerate(starts):
                en = starts[bi + 1] if bi + 1 < len(starts) else len(nodes)
                self.emit(f"if _pc <= {bi}:", ind + 2)
                self.emit("pass", ind + 3)
                for nd in nodes[st:en]:
                    self.node(nd, ind + 3)
            self.emit("break", ind + 2)
            self.emit("except _Goto as _g:", ind + 1)
            mapping = {nodes[st][1]: bi for bi, st in enumerate(starts) if nodes[st][1] is not None}
            self.emit(f"_pc = {self.bind(mapping, 'lab')}.get(_g.label)", ind + 2)
            self.emit("if _pc is None: raise", ind + 2)
            return
        if not nodes:
            self.emit("pass", ind)
        for nd in nodes:
            self.node(nd, ind)

    def node(self, nd, ind):
        k = nd[0]
        try:
            if k == "s":
                mark = len(self.lines)
                try:
                    self.stmt(nd[2], ind)
                except NotImplementedError as e:
                    # a statement outside the subset (string building for
                    # output file names, system calls): an error only if
                    # it is executed
                    del self.lines[mark:]
                    msg = f"{self.unit.path}:{nd[-1]}: {e}"
                    self.emit(f"raise NotImplementedError({msg!r})", ind)
            elif k == "if":
                _, lab, arms, els, n = nd
                for i, (cond, blk) in enumerate(arms):
                    c, t, _ = self.ex(parse_expr(cond))
                    self.emit(f"{'if' if i == 0 else 'elif'} {c}:", ind)
                    self.block(blk, ind + 1)
                if els is not None:
                    self.emit("else:", ind)
                    self.block(els, ind + 1)
            elif k == "select":
                _, lab, expr, arms, n = nd
                c, t, _ = self.ex(parse_expr(expr))
                v = f"_sel{n}"
                self.emit(f"{v} = {c}", ind)
                first, default = True, None
                for sel, blk in arms:
                    if sel is None:
                        default = blk
                        continue
                    tests = []
                    for item in sel:
                        if ":" in item:
                            lo, hi = (x.strip() for x in item.split(":", 1))
                            parts = ([f"{v} >= {self.ex(parse_expr(lo))[0]}"] if lo else []) + \
                                    ([f"{v} <= {self.ex(parse_expr(hi))[0]}"] if hi else [])
                            tests.append("(" + " and ".join(parts) + ")")
                        else:
                            tests.append(f"{v} == {self.ex(parse_expr(item))[0]}")
                    self.emit(f"{'if' if first else 'elif'} {' or '.join(tests)}:", ind)
                    self.block(blk, ind + 1)
                    first = False
                if default is not None:
                    if first:
                        self.block(default, ind)
                    else:
                        self.emit("else:", ind)
                        self.block(default, ind + 1)
            elif k == "while":
                _, lab, cond, blk, n = nd
                c, t, _ = self.ex(parse_expr(cond))
                self.emit(f"while {c}:", ind)
                self.block(blk, ind + 1)
            elif k == "do":
                self.do(nd, ind)
        except (NotImplementedError, SyntaxError, NameError) as e:
            raise type(e)(f"{self.unit.path}:{nd[-1]}: {e}") from e

    def do(self, nd, ind):
        _, lab, var, rng, blk, endl, n = nd
        lo = self.ex(parse_expr(rng[0]))
        hi = self.ex(parse_expr(rng[1]))
        st = self.ex(parse_expr(rng[2])) if len(rng) > 2 else ("1", "i4", False)
        kind, sym, ref = self.resolve(var)
        if sym is None or sym.t not in ("i4", "i8"):
            raise NotImplementedError(f"DO variable {var} must be an integer")
        tl, th, ts = self.newtmp(), self.newtmp(), self.newtmp()
        self.emit(f"{tl} = {self.conv(lo[0], lo[1], 'i8')}; {th} = {self.conv(hi[0], hi[1], 'i8')}; "
                  f"{ts} = {self.conv(st[0], st[1], 'i8')}", ind)
        it = self.newtmp()
        target = f"r_{var}" if var in self.regs else f"{ref}[0]"
        self.emit(f"for {it} in range({tl}, {tl} + _trip({tl}, {th}, {ts}) * {ts}, {ts}):", ind)
        self.emit(f"{target} = {it}", ind + 1)
        cyc = endl is not None and endl in self.goto_labels
        if cyc:
            self.emit("try:", ind + 1)
            self.block(blk, ind + 2)
            self.emit("except _Goto as _g:", ind + 1)
            self.emit(f"if _g.label != {endl}: raise", ind + 2)
        else:
            self.block(blk, ind + 1)
        self.emit(f"{target} = {tl} + _trip({tl}, {th}, {ts}) * {ts}", ind)

    def stmt(self, s, ind):
        m = re.match(r"^(open|close)\s*\(", s)
        if m:
            ctl = split_top(s[s.index("(") + 1:match_paren(s, s.index("("))])
            unit = next((c for c in ctl if "=" not in c), None)
            unit = unit or next(c.split("=", 1)[1] for c in ctl if c.split("=", 1)[0].strip() == "unit")
            if m.group(1) == "close":
                self.emit(f"_rt.io_close({self.int_ex(parse_expr(unit))})", ind)
                return
            f = next((c.split("=", 1)[1].strip() for c in ctl if c.split("=", 1)[0].strip() == "file"), None)
            if f and f[0] in "'\"" and f[-1] == f[0]:
                self.emit(f"_rt.io_open({self.int_ex(parse_expr(unit))}, {f[1:-1]!r})", ind)
            else:
                self.emit("pass", ind)
            return
        if s in ("continue",) or re.match(r"^(write|print|format|flush|inquire|rewind|backspace)\b", s):
            self.emit("pass", ind)
            return
        m = re.match(r"^if\s*\(", s)
        if m:
            j = match_paren(s, s.index("("))
            cond, rest = s[s.index("(") + 1:j], s[j + 1:].strip()
            c, t, _ = self.ex(parse_expr(cond))
            self.emit(f"if {c}:", ind)
            self.stmt(rest, ind + 1)
            return
        m = re.match(r"^go\s*to\s*(\d+)$", s)
        if m:
            self.emit(f"raise _Goto({int(m.group(1))})", ind)
            return
        if s == "return":
            self.emit(self.return_code(), ind)
            return
        m = re.match(r"^(?:stop|pause)\b\s*(.*)$", s)
        if m:
            self.emit(f"raise _Stop({m.group(1)!r})", ind)
            return
        m = re.match(r"^call\s+(\w+)\s*(\((.*)\))?$", s)
        if m:
            name = m.group(1)
            args = [] if not m.group(2) else _P(tokenize(m.group(2))).primary_args()
            kind, sym, ref = self.resolve(name)
            self.emit(self.call_code(name, args, kind == "dummy"), ind)
            return
        if s == "cycle":
            self.emit("continue", ind)
            return
        if s == "exit":
            self.emit("break", ind)
            return
        m = re.match(r"^(allocate|deallocate)\s*\((.*)\)$", s)
        if m:
            for item in split_top(m.group(2)):
                if "=" in item and item.split("=")[0].strip() in ("stat", "errmsg"):
                    continue
                if m.group(1) == "deallocate":
                    kind, sym, ref = self.resolve(item.strip())
                    self.emit(f"{ref} = None", ind)
                    continue
                nm = item[:item.index("(")].strip()
                dims = self.sc._dims(item[item.index("(") + 1:item.rindex(")")])
                kind, sym, ref = self.resolve(nm)
                lbs = [("1" if lo is None else self.int_ex(lo)) for lo, hi in dims]
                exts = [f"({self.int_ex(hi)})-({l})+1" for (lo, hi), l in zip(dims, lbs)]
                self.emit(f"{ref} = _FArr(np.zeros(({', '.join(exts)},), _DT[{sym.t!r}], order='F'), "
                          f"({', '.join(lbs)},), {sym.t!r})", ind)
            return
        if re.match(r"^read\s*\(", s):
            i = s.index("(")
            j = match_paren(s, i)
            ctl = split_top(s[i + 1:j])
            if len(ctl) != 2 or ctl[1].strip() != "*":
                raise NotImplementedError(f"READ other than list-directed: {s!r}")
            items = split_top(s[j + 1:].strip()) if s[j + 1:].strip() else []
            if any(it.strip().startswith("(") for it in items):
                raise NotImplementedError(f"implied DO in READ: {s!r}")
            self.emit(f"_v = _rt.io_read({self.int_ex(parse_expr(ctl[0]))}, {len(items)})", ind)
            for q, it in enumerate(items):
                le = parse_expr(it.strip())
                kind, sym, ref = self.resolve(le[1])
                if sym is None:
                    raise NameError(f"{self.unit.name}: unknown name {le[1]}")
                self.assign(le, it, f"_from_text(_v[{q}], {sym.t!r})", sym.t, False, ind)
            return
        # assignment
        i = _assign_split(s)
        if i is None:
            raise NotImplementedError(f"statement {s!r}")
        lhs, rhs = s[:i].strip(), s[i + 1:].strip()
        le = parse_expr(lhs)
        c, t, arr = self.ex(parse_expr(rhs))
        self.assign(le, lhs, c, t, arr, ind)

    def assign(self, le, lhs, c, t, arr, ind):
        """Store the value c (type t, an array if arr) in the variable,
        element or section le."""
        if le[0] == "name":
            kind, sym, ref = self.resolve(le[1])
            if kind is None:
                raise NameError(f"{self.unit.name}: unknown name {le[1]}")
            if sym.dims is not None:
                self.emit(f"{ref}.a[...] = {self.arr_conv(c, t, sym.t, arr)}", ind)
            elif le[1] in self.regs:
                self.emit(f"r_{le[1]} = {self.conv(c, t, sym.t)}", ind)
            else:
                self.emit(f"{ref}[0] = {self.conv(c, t, sym.t)}", ind)
            return
        if le[0] == "call":
            kind, sym, ref = self.resolve(le[1])
            if sym is None or sym.dims is None:
                raise NotImplementedError(f"assignment to {lhs}")
            idx, isarr = self.index_code(ref, sym, le[2])
            if isarr:
                self.emit(f"{ref}.a[{idx}] = {self.arr_conv(c, t, sym.t, arr)}", ind)
            else:
                self.emit(f"{ref}.a[{idx}] = {self.conv(c, t, sym.t)}", ind)
            return
        raise NotImplementedError(f"assignment to {lhs!r}")

    def arr_conv(self, c, t, to, arr):
        if not arr:
            return self.conv(c, t, to)
        if t == to:
            return c
        if to in ("r8",) and t in ("c8", "c16"):
            return f"np.real({c})"
        return c  # numpy casts on assignment (integer targets truncate)


def _if_then(s):
    i = s.index("(")
    j = match_paren(s, i)
    return s[j + 1:].strip() == "then"


def _assign_split(s):
    """Index of the assignment '=' of a statement, or None."""
    depth, q = 0, None
    for i, ch in enumerate(s):
        if q:
            if ch == q:
                q = None
            continue
        if ch in "'\"":
            q = ch
        elif ch == "(":
            depth += 1
        elif ch == ")":
            depth -= 1
        elif ch == "=" and depth == 0:
            if s[i + 1:i + 2] == "=" or s[i - 1:i] in "<>/=":
                continue
            return i
    return None


def _share_do_labels(tree):
    return tree


def _primary_args(self):
    args = []
    if self.peek()[1] != ")":
        while True:
            args.append(self.arg())
            if self.peek()[1] == ",":
                self.take()
                continue
            break
    self.take(")")
    return args


def _primary_args_entry(self):
    self.take("(")
    return _primary_args(self)


_P.primary_args = _primary_args_entry


# translated-code helpers
def _scalar_arg(a, t):
    if isinstance(a, Seq):
        f = a.flat
        if f.dtype != _DT[t]:
            raise TypeError(f"scalar argument of type {f.dtype} for a dummy of type {t}")
        return f[0:1]
    if isinstance(a, np.ndarray):
        return a.reshape(-1)[0:1]
    return np.array([a], _DT[t])


def _array_arg(a, t, lbs, exts):
    if isinstance(a, Seq):
        flat = a.flat
    elif isinstance(a, np.ndarray):
        flat = a.reshape(-1)
    else:
        raise TypeError("array dummy needs storage")
    if flat.dtype != _DT[t]:
        # storage association across types (a real array passed where a complex one is declared)
        flat = flat.view(_DT[t]) if flat.flags.c_contiguous else flat.copy().view(_DT[t])
    ext = flat
    if any(e is None for e in exts):
        n = flat.size
        shape = [int(e) for e in exts[:-1]]
        last = n // int(np.prod(shape)) if shape else n
        shape.append(last)
        flat = flat[:int(np.prod(shape))]
    else:
        shape = [int(e) for e in exts]
        n = int(np.prod(shape))
        if n > flat.size:
            raise IndexError(f"actual argument of {flat.size} elements for a dummy of {n}")
        flat = flat[:n]
    return FArr(flat.reshape(shape, order="F"), [int(l) for l in lbs], t, ext)


def _elem(arr, idx):
    off = arr.offset(idx)
    return Seq(arr.flat()[off:], arr.t)


def _section(a, t):
    if not (a.flags.f_contiguous or a.ndim <= 1 and a.flags.c_contiguous):
        raise NotImplementedError("non-contiguous array section as an actual argument")
    return Seq(a.reshape(-1, order="F"), t)


def _view(buf, off, t, shape):
    return view_bytes(buf, off, t, shape)


def _idiv_arr(a, b):
    return np.trunc(np.asarray(a) / np.asarray(b)).astype(np.asarray(a).dtype)


class _Stop(FortranStop):
    pass


_GLOBALS = {"np": np, "_math": math, "_cmath": __import__("cmath"), "_f32": np.float32, "_c64": np.complex64,
            "_DT": _DT, "_Seq": Seq, "_FArr": FArr, "_idiv": _idiv, "_idiv_arr": _idiv_arr, "_powi": _powi,
            "_fint": _fint, "_nint": _nint, "_aint": _aint, "_sign": _sign, "_mod": _mod, "_trip": _trip,
            "_Goto": _Goto, "_Stop": _Stop, "_scalar_arg": _scalar_arg, "_array_arg": _array_arg,
            "_elem": _elem, "_section": _section, "_view": _view, "_view_rest": view_rest}


def _from_text(tok, t):
    """A list-directed input value for a variable of type t."""
    if t in ("i4", "i8"):
        return int(tok)
    if t in ("r4", "r8"):
        v = float(tok.replace("d", "e").replace("D", "E"))
        return float(np.float32(v)) if t == "r4" else v
    if t == "l":
        return tok.lstrip(".").upper().startswith("T")
    raise NotImplementedError(f"list-directed READ into type {t}")


_GLOBALS["_from_text"] = _from_text


def translate(rt, unit):
    return Translator(rt, unit).translate()
