"""Minimal interpreter for the Fortran 90 subset used by the FWI solver files.

Used only to generate the golden vectors under tests/golden/ from the
reference's own source (no Fortran compiler exists in the build container).
It executes the reference subroutines as written, with default REAL as IEEE
single precision (numpy float32, one rounding per operation, no fused
multiply-add, no reassociation: what gfortran emits for x86-64 without
-march flags), default INTEGER as Python int, ``x**2`` as ``x*x`` and
``exp``/``log`` through the C library's ``expf``/``logf``.

Supported: subroutines and functions, internal procedures after CONTAINS
(host association), type declarations (explicit-shape, assumed-size,
allocatable; INTEGER, REAL, DOUBLE PRECISION, COMPLEX, LOGICAL, with or
without KIND=), allocate/deallocate, scalar/array/section/vector-subscript
assignment, DO / DO WHILE / IF blocks, one-line IF, CALL with
pass-by-reference (dummies alias the actual argument; explicit-shape and
assumed-size dummies are reshaped views, i.e. sequence association, also
from an array element onward and between COMPLEX actuals and REAL dummies,
which see the interleaved real and imaginary parts), EXIT/CYCLE/RETURN, and
the intrinsics these sources use.  I/O statements (write/print/open/close)
are skipped; READ is rejected.

COMPLEX arithmetic follows what gfortran emits (GCC's complex lowering under
-fcx-fortran-rules): an operand known to be real is combined componentwise
(r*(c,d) = (r*c, r*d), (a,b)/r = (a/r, b/r), r+(c,d) = (r+c, d)); complex
products are (ac - bd, ad + bc); a complex divisor uses the scaled division
of GCC's wide-range method (ratio = the smaller over the larger component of
the divisor); each operation rounded to single precision, x**2 = x*x.
Procedures that stand outside the executed sources (a trace reader, a
forward solver) can be supplied as Python callables (``natives``).
"""
from __future__ import annotations

import ctypes
import ctypes.util
import math
import re

import numpy as np

_libm = ctypes.CDLL(ctypes.util.find_library("m"))
_libm.expf.restype = ctypes.c_float
_libm.expf.argtypes = [ctypes.c_float]
_libm.logf.restype = ctypes.c_float
_libm.logf.argtypes = [ctypes.c_float]
for _f in ("cosf", "sinf", "atanf"):
    getattr(_libm, _f).restype = ctypes.c_float
    getattr(_libm, _f).argtypes = [ctypes.c_float]
C64 = np.complex64

F32 = np.float32


def _vec(fn, x):
    if isinstance(x, np.ndarray):
        out = np.empty(x.shape, dtype=np.float32, order="F")
        flat_in = x.reshape(-1, order="F")
        flat_out = out.reshape(-1, order="F")
        for i in range(flat_in.size):
            flat_out[i] = fn(float(flat_in[i]))
        return out
    return F32(fn(float(x)))


class Return(Exception):
    pass


class Exit(Exception):
    pass


class Cycle(Exception):
    pass


class Var:
    """A mutable box so that dummies can alias actual arguments."""

    __slots__ = ("value", "ftype", "alloc")

    def __init__(self, value=None, ftype="real", alloc=False):
        self.value = value
        self.ftype = ftype
        self.alloc = alloc


# ----------------------------------------------------------------------------
# lexing
# ----------------------------------------------------------------------------

def _strip_comment(line: str) -> str:
    out, q = [], None
    for ch in line:
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
        out.append(ch)
    return "".join(out)


def _split_semis(line: str):
    parts, depth, q, cur = [], 0, None, []
    for ch in line:
        if q:
            cur.append(ch)
            if ch == q:
                q = None
            continue
        if ch in "'\"":
            q = ch
        elif ch == "(":
            depth += 1
        elif ch == ")":
            depth -= 1
        elif ch == ";" and depth == 0:
            parts.append("".join(cur))
            cur = []
            continue
        cur.append(ch)
    parts.append("".join(cur))
    return [p.strip() for p in parts if p.strip()]


def logical_lines(text: str, with_labels: bool = False):
    """Yield (lineno, statement) pairs -- (lineno, statement, label) with
    with_labels -- with comments, continuations and statement labels removed,
    lower-cased."""
    raw = text.split("\n")
    buf, start = "", None
    for no, line in enumerate(raw, 1):
        s = _strip_comment(line).rstrip()
        if not s.strip():
            if buf:
                continue
            continue
        st = s.strip()
        if buf:
            if st.startswith("&"):
                st = st[1:]
            buf += " " + st
        else:
            buf, start = st, no
        if buf.endswith("&"):
            buf = buf[:-1]
            continue
        full = buf
        buf = ""
        ml = re.match(r"^(\d+)\s+", full)  # statement label
        label = int(ml.group(1)) if ml else None
        full = full[ml.end():] if ml else full
        for stmt in _split_semis(full):
            if with_labels:
                yield start, stmt.lower(), label
            else:
                yield start, stmt.lower()
            label = None


_TOKEN = re.compile(
    r"""
    (?P<ws>\s+)
  | (?P<str>'[^']*'|"[^"]*")
  | (?P<real>(\d+\.(?!(eq|ne|lt|le|gt|ge|and|or|not|true|false)\.)\d*([ed][+-]?\d+)?)|(\.\d+([ed][+-]?\d+)?)|(\d+[ed][+-]?\d+))
  | (?P<int>\d+)
  | (?P<dotop>\.(eq|ne|lt|le|gt|ge|and|or|not|true|false|eqv|neqv)\.)
  | (?P<name>[a-z_][a-z0-9_]*)
  | (?P<op>\*\*|//|==|/=|<=|>=|=>|[-+*/(),:<>=%])
    """,
    re.X,
)


def tokenize(s: str):
    pos, out = 0, []
    while pos < len(s):
        m = _TOKEN.match(s, pos)
        if not m:
            raise SyntaxError(f"cannot tokenize {s[pos:]!r} in {s!r}")
        pos = m.end()
        kind = m.lastgroup
        if kind == "ws":
            continue
        val = m.group(kind)
        if kind == "dotop":
            val = val.strip(".")
            mp = {"eq": "==", "ne": "/=", "lt": "<", "le": "<=", "gt": ">", "ge": ">="}
            if val in mp:
                out.append(("op", mp[val]))
            elif val in ("true", "false"):
                out.append(("bool", val == "true"))
            else:
                out.append(("op", "." + val + "."))
            continue
        out.append((kind, val))
    out.append(("end", None))
    return out


# ----------------------------------------------------------------------------
# expression parsing (Pratt)
# ----------------------------------------------------------------------------

_BIN = {
    ".or.": (1, "l"), ".and.": (2, "l"), ".eqv.": (0, "l"), ".neqv.": (0, "l"),
    "==": (4, "l"), "/=": (4, "l"), "<": (4, "l"), "<=": (4, "l"), ">": (4, "l"), ">=": (4, "l"),
    "//": (4.5, "l"),
    "+": (5, "l"), "-": (5, "l"),
    "*": (6, "l"), "/": (6, "l"),
    "**": (8, "r"),
}


class Parser:
    def __init__(self, toks):
        self.t = toks
        self.i = 0

    def peek(self):
        return self.t[self.i]

    def next(self):
        tok = self.t[self.i]
        self.i += 1
        return tok

    def expect(self, kind, val=None):
        tok = self.next()
        if tok[0] != kind or (val is not None and tok[1] != val):
            raise SyntaxError(f"expected {kind} {val}, got {tok}")
        return tok

    def expr(self, rbp=0):
        tok = self.next()
        left = self.nud(tok)
        while True:
            tok = self.peek()
            if tok[0] != "op" or tok[1] not in _BIN:
                break
            lbp, assoc = _BIN[tok[1]]
            if lbp <= rbp:
                break
            self.next()
            right = self.expr(lbp - 0.1 if assoc == "r" else lbp)
            left = ("bin", tok[1], left, right)
        return left

    def nud(self, tok):
        kind, val = tok
        if kind == "int":
            return ("int", int(val))
        if kind == "real":
            return ("real", F32(float(val.replace("d", "e"))))
        if kind == "bool":
            return ("bool", val)
        if kind == "str":
            return ("str", val[1:-1])
        if kind == "op" and val in ("-", "+"):
            # unary sign applies to a multiplication-level operand
            operand = self.expr(5)
            return ("neg", operand) if val == "-" else operand
        if kind == "op" and val == ".not.":
            return ("not", self.expr(3))
        if kind == "op" and val == "(":
            e = self.expr(0)
            if self.peek() == ("op", ","):  # complex constant (re, im)
                self.next()
                im = self.expr(0)
                self.expect("op", ")")
                return ("cplx", e, im)
            self.expect("op", ")")
            return ("paren", e)
        if kind == "name":
            if self.peek() == ("op", "("):
                self.next()
                args = []
                if self.peek() != ("op", ")"):
                    while True:
                        args.append(self.subscript())
                        if self.peek() == ("op", ","):
                            self.next()
                            continue
                        break
                self.expect("op", ")")
                return ("ref", val, args)
            return ("name", val)
        raise SyntaxError(f"unexpected token {tok}")

    def subscript(self):
        # range a:b, :, a:, :b, or expression; also keyword arg name=expr
        if self.peek() == ("op", ":"):
            self.next()
            hi = None
            if self.peek() not in (("op", ","), ("op", ")")):
                hi = self.expr(0)
            return ("range", None, hi)
        if self.peek()[0] == "name" and self.t[self.i + 1] == ("op", "="):
            name = self.next()[1]
            self.next()
            return ("kw", name, self.expr(0))
        e = self.expr(0)
        if self.peek() == ("op", ":"):
            self.next()
            hi = None
            if self.peek() not in (("op", ","), ("op", ")")):
                hi = self.expr(0)
            return ("range", e, hi)
        return e


def parse_expr(s: str):
    p = Parser(tokenize(s))
    e = p.expr(0)
    if p.peek()[0] != "end":
        raise SyntaxError(f"trailing tokens in {s!r}: {p.t[p.i:]}")
    return e


# ----------------------------------------------------------------------------
# statements
# ----------------------------------------------------------------------------

def _top_level_eq(s: str):
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
            prev = s[i - 1] if i else ""
            nxt = s[i + 1] if i + 1 < len(s) else ""
            if prev in "=/<>" or nxt in "=>":
                continue
            return i
    return -1


def _match_paren(s: str, start: int) -> int:
    depth = 0
    for i in range(start, len(s)):
        if s[i] == "(":
            depth += 1
        elif s[i] == ")":
            depth -= 1
            if depth == 0:
                return i
    raise SyntaxError(f"unbalanced parentheses in {s!r}")


_DECL = re.compile(r"^(?P<base>integer(\*\d+)?|real(\*\d+)?|complex(\*\d+)?|logical|character(\s*\([^)]*\))?(\*\d+)?"
                   r"|double\s+precision)\b(?P<rest>.*)$")
_KIND = re.compile(r"^(integer|real|complex|logical)\s*\(\s*kind\s*=\s*(\d+)\s*\)")


def _kind_spec(m):
    t, k = m.group(1), int(m.group(2))
    if t == "real" and k == 8:
        return "real*8"
    if t == "complex" and k == 8:
        return "complex*16"
    return t
_SKIP = re.compile(r"^(write|print|open|close|format|inquire|rewind)\b")


def _split_top(s: str, sep=","):
    parts, depth, cur = [], 0, []
    for ch in s:
        if ch == "(":
            depth += 1
        elif ch == ")":
            depth -= 1
        if ch == sep and depth == 0:
            parts.append("".join(cur).strip())
            cur = []
        else:
            cur.append(ch)
    if "".join(cur).strip():
        parts.append("".join(cur).strip())
    return parts


def parse_stmt(no, s):
    """Return a statement node."""
    if _SKIP.match(s):
        return ("skip", no)
    if s.startswith("read") and re.match(r"^read\s*\(", s):
        return ("read", no)
    if s == "continue":
        return ("continue", no)
    m = re.match(r"^go\s*to\s+(\d+)$", s)
    if m:
        return ("goto", no, int(m.group(1)))
    m = re.match(r"^equivalence\s*(\(.*\))$", s)
    if m:
        groups = [[n.strip() for n in g.split(",")] for g in re.findall(r"\(([^()]*)\)", m.group(1))]
        return ("equiv", no, groups)
    if re.match(r"^(implicit|use|include|save|intrinsic|external)\b", s):
        return ("skip", no)
    if s == "contains":
        return ("contains", no)
    s = _KIND.sub(_kind_spec, s)
    m = _DECL.match(s)
    if m:
        if True:
            base = m.group("base").replace(" ", "")
            rest = m.group("rest")
            attrs = ""
            if "::" in rest:
                attrs, ents = rest.split("::", 1)
            else:
                ents = rest
            ftype = "integer" if base.startswith("integer") else (
                "real" if base.startswith("real") and base in ("real", "real*4") else (
                    "double" if base in ("real*8", "doubleprecision") else (
                        "complex" if base in ("complex", "complex*8") else (
                            "logical" if base == "logical" else "character"))))
            alloc = "allocatable" in attrs
            # a DIMENSION(...) attribute gives every entity without its own
            # bounds that shape
            attr_dims = None
            md = re.search(r"dimension\s*\(", attrs)
            if md:
                start = md.end() - 1
                end = _match_paren(attrs, start)
                attr_dims = [d.strip() for d in _split_top(attrs[start + 1:end])]
                attr_dims = [None if d == ":" else (("star",) if d == "*" else parse_expr(d)) for d in attr_dims]
            entities = []
            for ent in _split_top(ents):
                ent = ent.strip()
                if not ent:
                    continue
                if "=" in ent and "(" not in ent.split("=")[0]:
                    name, init = ent.split("=", 1)
                    entities.append((name.strip(), None, parse_expr(init)))
                    continue
                mm = re.match(r"^([a-z_][a-z0-9_]*)\s*(\((.*)\))?\s*(\*\s*\d+)?$", ent)
                if not mm:
                    raise SyntaxError(f"bad declaration entity {ent!r}")
                dims = attr_dims
                if mm.group(2):
                    dims = [d.strip() for d in _split_top(mm.group(3))]
                    dims = [None if d == ":" else (("star",) if d == "*" else parse_expr(d)) for d in dims]
                entities.append((mm.group(1), dims, None))
            return ("decl", no, ftype, alloc, entities)
    if s in ("return",):
        return ("return", no)
    if s in ("exit",):
        return ("exit", no)
    if s in ("cycle",):
        return ("cycle", no)
    if s.startswith("stop"):
        return ("stop", no)
    m = re.match(r"^(allocate|deallocate)\s*\((.*)\)$", s)
    if m:
        items = []
        for it in _split_top(m.group(2)):
            mm = re.match(r"^([a-z_][a-z0-9_]*)\s*(\((.*)\))?$", it.strip())
            if not mm:
                continue  # stat= etc.
            dims = None
            if mm.group(2):
                dims = []
                for d in _split_top(mm.group(3)):
                    lo_hi = _split_top(d, ":")
                    if len(lo_hi) == 2:
                        if lo_hi[0].strip() != "1":
                            raise SyntaxError(f"line {no}: lower bound other than 1 in {s!r}")
                        d = lo_hi[1]
                    dims.append(parse_expr(d))
            items.append((mm.group(1), dims))
        return (m.group(1), no, items)
    m = re.match(r"^call\s+([a-z_][a-z0-9_]*)\s*(\((.*)\))?$", s)
    if m:
        args = []
        if m.group(2):
            p = Parser(tokenize(m.group(3)))
            if p.peek()[0] != "end":
                while True:
                    args.append(p.subscript())
                    if p.peek() == ("op", ","):
                        p.next()
                        continue
                    break
        return ("call", no, m.group(1), args)
    if s == "do":
        return ("dowhile", no, ("bool", True))
    m = re.match(r"^do\s+while\s*\((.*)\)$", s)
    if m:
        return ("dowhile", no, parse_expr(m.group(1)))
    m = re.match(r"^do\s+(\d+)\s*,?\s*([a-z_][a-z0-9_]*)\s*=\s*(.*)$", s)
    if m:  # DO <label> var = ...: the loop ends at the labelled statement
        parts = _split_top(m.group(3))
        return ("dolab", no, int(m.group(1)), m.group(2), [parse_expr(p) for p in parts])
    m = re.match(r"^do\s+([a-z_][a-z0-9_]*)\s*=\s*(.*)$", s)
    if m:
        parts = _split_top(m.group(2))
        return ("do", no, m.group(1), [parse_expr(p) for p in parts])
    if s in ("enddo", "end do"):
        return ("enddo", no)
    if s in ("endif", "end if"):
        return ("endif", no)
    if s == "else":
        return ("else", no)
    m = re.match(r"^else\s*if\s*\(", s)
    if m:
        i0 = s.index("(")
        i1 = _match_paren(s, i0)
        return ("elseif", no, parse_expr(s[i0 + 1:i1]))
    if s.startswith("if") and re.match(r"^if\s*\(", s):
        i0 = s.index("(")
        i1 = _match_paren(s, i0)
        cond = parse_expr(s[i0 + 1:i1])
        rest = s[i1 + 1:].strip()
        if rest == "then":
            return ("ifthen", no, cond)
        return ("if1", no, cond, parse_stmt(no, rest))
    if re.match(r"^end(\s*(subroutine|function|program)\b.*)?$", s):
        return ("end", no)
    k = _top_level_eq(s)
    if k > 0:
        lhs = parse_expr(s[:k])
        rhs = parse_expr(s[k + 1:])
        return ("assign", no, lhs, rhs)
    raise SyntaxError(f"line {no}: cannot parse statement {s!r}")


def build_blocks(stmts):
    """Turn a flat statement list into nested blocks."""
    pos = 0

    def block(terminators):
        nonlocal pos
        body = []
        while pos < len(stmts):
            st = stmts[pos]
            kind = st[0]
            if kind in terminators:
                return body
            pos += 1
            if kind == "do" or kind == "dowhile":
                inner = block({"enddo"})
                pos += 1
                body.append(st + (inner,))
            elif kind == "ifthen":
                branches = []
                cond = st[2]
                while True:
                    inner = block({"elseif", "else", "endif"})
                    branches.append((cond, inner))
                    term = stmts[pos]
                    pos += 1
                    if term[0] == "endif":
                        break
                    if term[0] == "elseif":
                        cond = term[2]
                    else:
                        cond = ("bool", True)
                body.append(("ifblock", st[1], branches))
            else:
                body.append(st)
        return body

    out = block(set())
    return out


class Unit:
    def __init__(self, kind, name, args, body, decls, result=None):
        self.kind, self.name, self.args, self.body, self.decls, self.result = kind, name, args, body, decls, result


def _make_unit(cur, stmts, labels, implicit_none):
    decls = [x for x in stmts if x[0] == "decl"]
    equivs = [g for x in stmts if x[0] == "equiv" for g in x[2]]
    rest = [(x, lab) for x, lab in zip(stmts, labels) if x[0] not in ("decl", "equiv")]
    flat = any(x[0] in ("goto", "dolab") or (x[0] == "if1" and x[3][0] == "goto") for x, _ in rest)
    body = [] if flat else build_blocks([x for x, _ in rest])
    u = Unit(cur[0], cur[1], cur[2], body, decls)
    u.implicit = not implicit_none
    u.equivs = equivs
    u.flat = rest if flat else None  # statements with labels, run by a program counter
    u.internals = {}
    u.host = None
    return u


def parse_units(text: str):
    units = {}
    cur = None
    stmts = []
    labels = []
    host = None  # a unit whose internal procedures (after CONTAINS) are being read
    for no, s, label in logical_lines(text, with_labels=True):
        m = re.match(r"^(?:(?:integer|real|logical)\s+)?(subroutine|function)\s+([a-z_][a-z0-9_]*)\s*(\((.*)\))?", s)
        if m and cur is None:
            args = [a.strip() for a in (m.group(4) or "").split(",") if a.strip()]
            cur = (m.group(1), m.group(2), args)
            stmts = []
            labels = []
            implicit_none = False
            continue
        if cur is None:
            if host is not None and re.match(r"^end(\s*(subroutine|function|program)\b.*)?$", s):
                hcur, hstmts, hlabels, himpl, internals = host
                u = _make_unit(hcur, hstmts, hlabels, himpl)
                u.internals = internals
                for iu in internals.values():
                    iu.host = u
                    iu.implicit = iu.implicit and not himpl
                units[hcur[1]] = u
                host = None
            continue  # module code, program code: not executed here
        if re.match(r"^implicit\s+none", s):
            implicit_none = True
        try:
            st = parse_stmt(no, s)
        except SyntaxError:
            st = ("bad", no, s)
        if st[0] == "contains" and host is None:
            host = (cur, stmts, labels, implicit_none, {})
            cur = None
            continue
        if st[0] == "end" and not _open_blocks(stmts):
            u = _make_unit(cur, stmts, labels, implicit_none)
            if host is not None:
                host[4][cur[1]] = u
            else:
                units[cur[1]] = u
            cur = None
            continue
        stmts.append(st)
        labels.append(label)
    return units


def _open_blocks(stmts):
    depth = 0
    for st in stmts:
        if st[0] in ("do", "dowhile", "ifthen"):
            depth += 1
        elif st[0] in ("enddo", "endif"):
            depth -= 1
    return depth > 0


# ----------------------------------------------------------------------------
# evaluation
# ----------------------------------------------------------------------------

def _is_int(x):
    if isinstance(x, (bool, np.bool_)):
        return False
    if isinstance(x, (int, np.integer)):
        return True
    return isinstance(x, np.ndarray) and x.dtype.kind in "iu"


def _to_real(x):
    if isinstance(x, np.ndarray):
        return x.astype(np.float32) if x.dtype != np.float32 and x.dtype != np.float64 else x
    if isinstance(x, (np.float32, np.float64)):
        return x
    return F32(x)


def _is_c(x):
    return isinstance(x, (complex, np.complexfloating)) or (isinstance(x, np.ndarray) and x.dtype.kind == "c")


def _cre(x):
    if _is_c(x):
        return x.real.astype(np.float32) if isinstance(x, np.ndarray) else F32(x.real)
    return _to_real(x)


def _cim(x):
    return x.imag.astype(np.float32) if isinstance(x, np.ndarray) else F32(x.imag)


def _cmk(re, im):
    if isinstance(re, np.ndarray) or isinstance(im, np.ndarray):
        re, im = np.broadcast_arrays(np.asarray(re, np.float32), np.asarray(im, np.float32))
        out = np.empty(re.shape, C64, order="F")
        out.real = re
        out.imag = im
        return out
    return C64(complex(float(re), float(im)))


def _cbin(op, a, b):
    """One COMPLEX operation as gfortran lowers it (see the module docstring):
    single-precision rounding of every real operation."""
    ca, cb = _is_c(a), _is_c(b)
    if op in ("+", "-"):
        f = (lambda x, y: x + y) if op == "+" else (lambda x, y: x - y)
        if ca and cb:
            return _cmk(f(_cre(a), _cre(b)), f(_cim(a), _cim(b)))
        if ca:
            return _cmk(f(_cre(a), _to_real(b)), _cim(a))
        return _cmk(f(_to_real(a), _cre(b)), _cim(b) if op == "+" else -_cim(b))
    if op == "*":
        if ca and cb:
            ar, ai, br, bi = _cre(a), _cim(a), _cre(b), _cim(b)
            return _cmk(ar * br - ai * bi, ar * bi + ai * br)
        if ca:
            r = _to_real(b)
            return _cmk(_cre(a) * r, _cim(a) * r)
        r = _to_real(a)
        return _cmk(r * _cre(b), r * _cim(b))
    if op == "/":
        if not cb:
            r = _to_real(b)
            return _cmk(_cre(a) / r, _cim(a) / r)
        ar = _cre(a)
        ai = _cim(a) if ca else (np.zeros_like(ar) if isinstance(ar, np.ndarray) else F32(0))
        br, bi = _cre(b), _cim(b)
        with np.errstate(all="ignore"):
            # |br| < |bi|: ratio = br/bi, else ratio = bi/br (GCC's wide-range division)
            r1 = br / bi
            d1 = br * r1 + bi
            t1r, t1i = ar * r1 + ai, ai * r1 - ar
            r2 = bi / br
            d2 = bi * r2 + br
            t2r, t2i = ai * r2 + ar, ai - ar * r2
            small = np.abs(br) < np.abs(bi)
            tr = np.where(small, t1r, t2r).astype(np.float32)
            ti = np.where(small, t1i, t2i).astype(np.float32)
            dv = np.where(small, d1, d2).astype(np.float32)
            re, im = tr / dv, ti / dv
        if not isinstance(re, np.ndarray) or re.ndim == 0:
            re, im = F32(re), F32(im)
        return _cmk(re, im)
    raise RuntimeError(f"operator {op} on COMPLEX operands")


def _int_div(a, b):
    if isinstance(a, np.ndarray) or isinstance(b, np.ndarray):
        q = np.abs(a) // np.abs(b)
        return np.where((np.sign(a) * np.sign(b)) < 0, -q, q)
    q = abs(a) // abs(b)
    return -q if (a < 0) != (b < 0) else q


def _power(a, b):
    if _is_int(b) or (isinstance(b, (np.float32, np.float64)) and float(b).is_integer()):
        n = int(b)
        if _is_int(a) and not isinstance(a, np.ndarray):
            return a ** n
        if n == 0:
            return np.ones_like(a) if isinstance(a, np.ndarray) else F32(1)
        if n < 0:
            return F32(1) / _power(a, -n)
        r = a
        # gfortran expands small integer powers by repeated multiplication
        for _ in range(n - 1):
            r = _cbin("*", r, a) if _is_c(a) else r * a
        return r
    return np.power(_to_real(a), _to_real(b))


class Interp:
    def __init__(self, units, globals_=None, overrides=None, natives=None):
        self.units = units
        self.globals = globals_ or {}
        self.overrides = overrides or {}
        self.natives = natives or {}

    def resolve(self, ctx, name):
        """(unit, host env) of a procedure called from ctx: an internal
        procedure of the calling unit or of its host, else a top-level one."""
        u = ctx["unit"]
        if name in getattr(u, "internals", {}):
            return u.internals[name], ctx["env"]
        host = getattr(u, "host", None)
        if host is not None and name in host.internals:
            return host.internals[name], ctx.get("host_env")
        if name in self.units:
            return self.units[name], None
        return None, None

    # -- entry ------------------------------------------------------------
    def call(self, name, actuals, unit=None, host_env=None):
        """Call a unit with a list of Var objects (by reference)."""
        u = unit if unit is not None else self.units[name]
        env = {}
        for dummy, act in zip(u.args, actuals):
            env[dummy] = act
        ctx = {"unit": u, "env": env, "implicit": getattr(u, "implicit", False), "host_env": host_env}
        # declarations: args first bound; now declare locals and reshape dummies
        for d in u.decls:
            _, no, ftype, alloc, entities = d
            for (nm, dims, init) in entities:
                if nm in env and nm in u.args:
                    v = env[nm]
                    if dims is not None and not alloc and isinstance(v.value, np.ndarray):
                        env[nm] = Var(self._dummy_view(ctx, name, nm, dims, ftype, v.value), ftype)
                    continue
                if nm == name and u.kind == "function":
                    env[nm] = Var(self._zero(ftype), ftype)
                    continue
                if alloc:
                    env[nm] = Var(None, ftype, alloc=True)
                elif dims is not None:
                    shape = self._dims(ctx, dims, None)
                    env[nm] = Var(np.zeros(shape, dtype=self._dtype(ftype), order="F"), ftype)
                else:
                    env[nm] = Var(self._zero(ftype) if init is None else self.eval(ctx, init), ftype)
        if u.kind == "function" and name not in env:
            env[name] = Var(F32(0), "real")
        # EQUIVALENCE: names of one group and of the same type share storage
        # (members of another type keep their own: they are only aliased in
        # memory, which these sources never read across types)
        for group in getattr(u, "equivs", []):
            first = {}
            for nm in group:
                v = self.lookup(ctx, nm)
                if v.ftype in first:
                    env[nm] = first[v.ftype]
                else:
                    first[v.ftype] = v
        try:
            if getattr(u, "flat", None) is not None:
                self.run_flat(ctx, u.flat)
            else:
                self.run(ctx, u.body)
        except Return:
            pass
        if u.kind == "function":
            return env[name].value
        return None

    def _dims(self, ctx, dims, actual):
        if any(d is None for d in dims):
            return None
        return [int(self.eval(ctx, d)) for d in dims]

    def _dummy_view(self, ctx, unit, nm, dims, ftype, arr):
        """The array dummy nm of the given declared shape (a trailing '*' takes
        the rest) over the storage of its actual: sequence association, from
        the actual's first element on; a COMPLEX actual seen by a REAL dummy
        is its interleaved real and imaginary parts."""
        flat = arr.reshape(-1, order="F")
        if arr.size and not np.shares_memory(flat, arr):
            raise RuntimeError(f"{unit}: non-contiguous actual for {nm}")
        want = self._dtype(ftype)
        if flat.dtype != want:
            if flat.dtype == C64 and want == np.float32:
                flat = flat.view(np.float32)
            else:
                raise RuntimeError(f"{unit}: actual of type {flat.dtype} for dummy {nm} of type {ftype}")
        shape = [None if d[0] == "star" else int(self.eval(ctx, d)) for d in dims]
        if None in shape:
            known = int(np.prod([x for x in shape if x is not None])) if len(shape) > 1 else 1
            shape = [x if x is not None else flat.size // max(known, 1) for x in shape]
        n = int(np.prod(shape))
        if n > flat.size:
            raise RuntimeError(f"{unit}: dummy {nm}{tuple(shape)} larger than its actual ({flat.size})")
        return flat[:n].reshape(tuple(shape), order="F")

    @staticmethod
    def _dtype(ftype):
        return {"integer": np.int64, "real": np.float32, "double": np.float64, "logical": np.bool_,
                "complex": C64}.get(ftype, np.float32)

    @staticmethod
    def _zero(ftype):
        return {"integer": 0, "real": F32(0), "double": np.float64(0), "logical": False,
                "complex": C64(0)}.get(ftype, None)

    # -- statements ---------------------------------------------------------
    def run_flat(self, ctx, flat):
        """Statements with labels, GO TO and labelled DO loops, run by a
        program counter (no block structure in these units)."""
        where = {lab: i for i, (_, lab) in enumerate(flat) if lab is not None}
        loops = []  # [var, iterations left, step, first body index, end index]
        pc = 0
        while pc < len(flat):
            st, _ = flat[pc]
            kind = st[0]
            nxt = pc + 1
            if kind == "dolab":
                _, no, endlab, var, parts = st
                lo = int(self.eval(ctx, parts[0]))
                hi = int(self.eval(ctx, parts[1]))
                step = int(self.eval(ctx, parts[2])) if len(parts) > 2 else 1
                count = max((hi - lo + step) // step, 0)
                v = self.lookup(ctx, var)
                v.value = lo
                if count == 0:
                    nxt = where[endlab] + 1
                else:
                    loops.append([v, count, step, pc + 1, where[endlab]])
            elif kind == "goto":
                nxt = where[st[2]]
            elif kind == "if1" and st[3][0] == "goto":
                if self.truth(self.eval(ctx, st[2])):
                    nxt = where[st[3][2]]
            elif kind in ("continue", "skip"):
                pass
            else:
                self.exec(ctx, st)
            if nxt == pc + 1:
                # the statement that ends a loop: next iteration or leave it
                while loops and loops[-1][4] == pc:
                    lp = loops[-1]
                    lp[1] -= 1
                    lp[0].value = lp[0].value + lp[2]
                    if lp[1] > 0:
                        nxt = lp[3]
                        break
                    loops.pop()
            else:
                while loops and not (loops[-1][3] <= nxt <= loops[-1][4]):
                    loops.pop()  # a jump out of the loop
            pc = nxt

    def run(self, ctx, body):
        for st in body:
            self.exec(ctx, st)

    def exec(self, ctx, st):
        kind = st[0]
        if kind == "assign":
            self.assign(ctx, st[2], st[3])
        elif kind == "do":
            _, no, var, parts, inner = st
            lo = int(self.eval(ctx, parts[0]))
            hi = int(self.eval(ctx, parts[1]))
            step = int(self.eval(ctx, parts[2])) if len(parts) > 2 else 1
            count = max((hi - lo + step) // step, 0)
            v = self.lookup(ctx, var)
            i = lo
            for _ in range(count):
                v.value = i
                try:
                    self.run(ctx, inner)
                except Cycle:
                    pass
                except Exit:
                    break
                i += step
            else:
                v.value = i
        elif kind == "dowhile":
            _, no, cond, inner = st
            while self.truth(self.eval(ctx, cond)):
                try:
                    self.run(ctx, inner)
                except Cycle:
                    continue
                except Exit:
                    break
        elif kind == "ifblock":
            for cond, inner in st[2]:
                if self.truth(self.eval(ctx, cond)):
                    self.run(ctx, inner)
                    break
        elif kind == "if1":
            if self.truth(self.eval(ctx, st[2])):
                self.exec(ctx, st[3])
        elif kind == "call":
            self.do_call(ctx, st[2], st[3])
        elif kind == "allocate":
            for nm, dims in st[2]:
                v = self.lookup(ctx, nm)
                shape = [int(self.eval(ctx, d)) for d in dims]
                v.value = np.zeros(shape, dtype=self._dtype(v.ftype), order="F")
        elif kind == "deallocate":
            for nm, _ in st[2]:
                self.lookup(ctx, nm).value = None
        elif kind == "return":
            raise Return()
        elif kind == "exit":
            raise Exit()
        elif kind == "cycle":
            raise Cycle()
        elif kind in ("skip", "continue"):
            pass
        elif kind == "bad":
            raise RuntimeError(f"line {st[1]}: statement not supported: {st[2]!r}")
        elif kind == "read":
            raise RuntimeError(f"READ statement at line {st[1]} is not supported")
        elif kind == "stop":
            raise RuntimeError(f"STOP at line {st[1]}")
        else:
            raise RuntimeError(f"unhandled statement {st}")

    def truth(self, v):
        return bool(v)

    def lookup(self, ctx, name):
        env = ctx["env"]
        if name in env:
            return env[name]
        host = ctx.get("host_env")
        if host is not None and name in host:
            return host[name]
        if name in self.globals:
            return self.globals[name]
        if ctx.get("implicit", True):
            # implicit typing (no IMPLICIT NONE in the unit): i-n integer, else real
            ftype = "integer" if name[0] in "ijklmn" else "real"
            env[name] = Var(self._zero(ftype), ftype)
            return env[name]
        raise NameError(f"{ctx['unit'].name}: unknown variable {name}")

    def has_var(self, ctx, name):
        host = ctx.get("host_env")
        return name in ctx["env"] or (host is not None and name in host) or name in self.globals

    # -- calls --------------------------------------------------------------
    def do_call(self, ctx, name, args):
        if name.startswith("mpi_"):
            # single-process stubs: rank 0 of 1; other MPI calls are no-ops
            if not getattr(self, "mpi_stub", False):
                raise RuntimeError("MPI call in interpreted code")
            if name in ("mpi_comm_size", "mpi_comm_rank"):
                self.lookup(ctx, args[1][1]).value = 1 if name == "mpi_comm_size" else 0
            return
        callee, host_env = self.resolve(ctx, name)
        array_dummy = set()
        if callee is not None:
            for d in callee.decls:
                for (nm, dims, init) in d[4]:
                    if nm in callee.args and dims is not None and not d[3]:
                        array_dummy.add(callee.args.index(nm))
        actuals, writeback = [], []
        for k, a in enumerate(args):
            if a[0] == "name" and self.has_var(ctx, a[1]):
                actuals.append(self.lookup(ctx, a[1]))
            elif a[0] == "ref" and self.has_var(ctx, a[1]):
                base = self.lookup(ctx, a[1])
                idx, basic, scalar = self.index(ctx, base.value, a[2])
                if scalar and k in array_dummy:
                    # an array element actual for an array dummy: the storage
                    # from that element on (sequence association)
                    off = int(np.ravel_multi_index(idx, base.value.shape, order="F"))
                    actuals.append(Var(base.value.reshape(-1, order="F")[off:], base.ftype))
                elif scalar:
                    box = Var(base.value[idx], base.ftype)
                    actuals.append(box)
                    writeback.append((base, idx, box))
                elif basic:
                    actuals.append(Var(base.value[idx], base.ftype))
                else:
                    actuals.append(Var(np.array(base.value[idx], order="F"), base.ftype))
            else:
                val = self.eval(ctx, a)
                ftype = "integer" if _is_int(val) else ("logical" if isinstance(val, (bool, np.bool_)) else "real")
                actuals.append(Var(val, ftype))
        if name in self.natives:
            self.natives[name](*actuals)
        elif callee is None:
            raise NameError(f"unknown subroutine {name}")
        else:
            self.call(name, actuals, unit=callee, host_env=host_env)
        for base, idx, box in writeback:
            base.value[idx] = box.value

    # -- assignment ---------------------------------------------------------
    def assign(self, ctx, lhs, rhs):
        val = self.eval(ctx, rhs)
        unit = ctx["unit"].name
        if lhs[0] == "name":
            v = self.lookup(ctx, lhs[1])
            key = (unit, lhs[1])
            if key in self.overrides:
                val = self.overrides[key]
            if isinstance(v.value, np.ndarray):
                if isinstance(val, np.ndarray) and val.shape != v.value.shape:
                    if v.alloc:
                        v.value = np.array(val, dtype=v.value.dtype, order="F")
                        return
                    raise RuntimeError(f"shape mismatch in assignment to {lhs[1]}")
                v.value[...] = self._conv(val, v.value.dtype)
            elif v.alloc and isinstance(val, np.ndarray):
                v.value = np.array(val, dtype=self._dtype(v.ftype), order="F")
            else:
                v.value = self._conv_scalar(val, v.ftype)
            return
        if lhs[0] == "ref":
            v = self.lookup(ctx, lhs[1])
            idx, basic, scalar = self.index(ctx, v.value, lhs[2])
            if scalar:
                v.value[idx] = self._conv(val, v.value.dtype)
            else:
                target_shape = v.value[idx].shape
                conv = self._conv(val, v.value.dtype)
                if isinstance(conv, np.ndarray) and conv.shape != target_shape:
                    conv = conv.reshape(target_shape, order="F")
                v.value[idx] = conv
            return
        raise RuntimeError(f"bad assignment target {lhs}")

    def _conv(self, val, dtype):
        if dtype.kind in "iu":
            if isinstance(val, np.ndarray):
                return np.trunc(val).astype(dtype) if val.dtype.kind == "f" else val.astype(dtype)
            return int(math.trunc(float(val))) if not _is_int(val) else val
        if dtype == C64:
            if _is_c(val):
                return val.astype(C64) if isinstance(val, np.ndarray) else C64(val)
            return _cmk(_to_real(val), F32(0))
        if dtype == np.float32:
            if _is_c(val):
                return _cre(val)
            return val.astype(np.float32) if isinstance(val, np.ndarray) else F32(val)
        return val

    def _conv_scalar(self, val, ftype):
        if ftype == "integer":
            return int(math.trunc(float(val))) if not _is_int(val) else int(val)
        if ftype == "real":
            return _cre(val) if _is_c(val) else F32(val)
        if ftype == "complex":
            return C64(val) if _is_c(val) else _cmk(_to_real(val), F32(0))
        if ftype == "double":
            return np.float64(val)
        if ftype == "logical":
            return bool(val)
        return val

    # -- indexing -----------------------------------------------------------
    def index(self, ctx, arr, subs):
        """Return (numpy index, is_basic, is_scalar_element)."""
        if arr is None:
            raise RuntimeError("indexing an unallocated array")
        parts, vec_dims, scalar = [], [], True
        for k, s in enumerate(subs):
            if s[0] == "range":
                lo = 1 if s[1] is None else int(self.eval(ctx, s[1]))
                hi = arr.shape[k] if s[2] is None else int(self.eval(ctx, s[2]))
                parts.append(slice(lo - 1, hi))
                scalar = False
            else:
                v = self.eval(ctx, s)
                if isinstance(v, np.ndarray):
                    parts.append(np.asarray(v, dtype=np.int64) - 1)
                    vec_dims.append(k)
                    scalar = False
                else:
                    iv = int(v)
                    if iv < 1 or iv > arr.shape[k]:
                        raise IndexError(f"{ctx['unit'].name}: subscript {iv} out of bounds 1..{arr.shape[k]}")
                    parts.append(iv - 1)
        if not vec_dims:
            for k, p in enumerate(parts):
                if isinstance(p, slice) and (p.start < 0 or p.stop > arr.shape[k]):
                    if p.stop > p.start:
                        raise IndexError(f"{ctx['unit'].name}: section {p} out of bounds")
            return tuple(parts), True, scalar
        # vector subscripts: build an open mesh over the non-scalar dims
        lists, keep = [], []
        for k, p in enumerate(parts):
            if isinstance(p, slice):
                lists.append(np.arange(p.start, p.stop))
                keep.append(True)
            elif isinstance(p, np.ndarray):
                if p.min() < 0 or p.max() >= arr.shape[k]:
                    raise IndexError("vector subscript out of bounds")
                lists.append(p)
                keep.append(True)
            else:
                lists.append(np.array([p]))
                keep.append(False)
        mesh = np.ix_(*lists)
        mesh = tuple(m if kp else m.reshape(m.shape) for m, kp in zip(mesh, keep))
        # squeeze scalar dims by taking index 0 along them afterwards
        return _MeshIndex(mesh, keep), False, False

    # -- expressions --------------------------------------------------------
    def eval(self, ctx, e):
        k = e[0]
        if k == "int":
            return e[1]
        if k == "real":
            return e[1]
        if k == "bool":
            return e[1]
        if k == "str":
            return e[1]
        if k == "paren":
            return self.eval(ctx, e[1])
        if k == "cplx":
            return _cmk(_to_real(self.eval(ctx, e[1])), _to_real(self.eval(ctx, e[2])))
        if k == "neg":
            v = self.eval(ctx, e[1])
            return -v
        if k == "not":
            return not self.eval(ctx, e[1])
        if k == "name":
            v = self.lookup(ctx, e[1])
            return v.value
        if k == "bin":
            return self.binop(e[1], self.eval(ctx, e[2]), self.eval(ctx, e[3]))
        if k == "ref":
            name, args = e[1], e[2]
            if self.has_var(ctx, name):
                v = self.lookup(ctx, name)
                if not isinstance(v.value, np.ndarray):
                    raise RuntimeError(f"{name} is not an array")
                idx, basic, scalar = self.index(ctx, v.value, args)
                out = v.value[idx]
                if isinstance(idx, _MeshIndex):
                    axes = tuple(i for i, kp in enumerate(idx.keep) if not kp)
                    if axes:
                        out = out.squeeze(axis=axes)
                if isinstance(out, np.ndarray):
                    return np.array(out, order="F")
                return out
            callee, host_env = self.resolve(ctx, name)
            if callee is not None:
                actuals = []
                for a in args:
                    if a[0] == "name" and self.has_var(ctx, a[1]):
                        actuals.append(self.lookup(ctx, a[1]))
                    else:
                        val = self.eval(ctx, a)
                        actuals.append(Var(val, "integer" if _is_int(val) else "real"))
                return self.call(name, actuals, unit=callee, host_env=host_env)
            return self.intrinsic(ctx, name, args)
        raise RuntimeError(f"cannot evaluate {e}")

    def binop(self, op, a, b):
        if op in ("+", "-", "*", "/") and (_is_c(a) or _is_c(b)):
            return _cbin(op, a, b)
        if op in ("+", "-", "*", "/"):
            if _is_int(a) and _is_int(b):
                if op == "+":
                    return a + b
                if op == "-":
                    return a - b
                if op == "*":
                    return a * b
                return _int_div(a, b)
            a, b = _to_real(a), _to_real(b)
            if op == "+":
                return a + b
            if op == "-":
                return a - b
            if op == "*":
                return a * b
            return a / b
        if op == "**":
            return _power(a, b)
        if op in ("==", "/=", "<", "<=", ">", ">="):
            if not (_is_int(a) and _is_int(b)):
                a, b = _to_real(a), _to_real(b)
            return {"==": a == b, "/=": a != b, "<": a < b, "<=": a <= b, ">": a > b, ">=": a >= b}[op]
        if op == ".and.":
            return bool(a) and bool(b)
        if op == ".or.":
            return bool(a) or bool(b)
        raise RuntimeError(f"operator {op}")

    def intrinsic(self, ctx, name, args):
        vals = [self.eval(ctx, a) for a in args if a[0] != "kw"]
        if name == "abs":
            return np.abs(vals[0]) if isinstance(vals[0], np.ndarray) else abs(vals[0])
        if name == "sqrt":
            return np.sqrt(_to_real(vals[0]))
        if name == "exp":
            return _vec(_libm.expf, _to_real(vals[0]))
        if name == "log":
            return _vec(_libm.logf, _to_real(vals[0]))
        if name in ("cos", "sin", "atan"):
            return _vec(getattr(_libm, name + "f"), _to_real(vals[0]))
        if name == "aimag":
            return _cim(vals[0])
        if name == "conjg":
            return _cmk(_cre(vals[0]), -_cim(vals[0]))
        if name == "cmplx":
            return _cmk(_to_real(vals[0]), _to_real(vals[1]) if len(vals) > 1 else F32(0))
        if name in ("maxval", "minval"):
            arr = vals[0]
            return arr.max() if name == "maxval" else arr.min()
        if name in ("real", "float"):
            return _cre(vals[0])
        if name == "int":
            v = vals[0]
            return np.trunc(v).astype(np.int64) if isinstance(v, np.ndarray) else int(math.trunc(float(v)))
        if name == "nint":
            return int(np.rint(vals[0]))
        if name == "ceiling":
            return int(math.ceil(float(vals[0])))
        if name == "floor":
            return int(math.floor(float(vals[0])))
        if name == "mod":
            a, b = vals
            if _is_int(a) and _is_int(b):
                return a - _int_div(a, b) * b
            return np.fmod(_to_real(a), _to_real(b))
        if name in ("max", "min"):
            if all(_is_int(v) for v in vals):
                return max(vals) if name == "max" else min(vals)
            vals = [_to_real(v) for v in vals]
            r = vals[0]
            for v in vals[1:]:
                r = np.maximum(r, v) if name == "max" else np.minimum(r, v)
            return r
        if name == "dot_product":
            a, b = _to_real(vals[0]), _to_real(vals[1])
            s = F32(0)
            for x, y in zip(a.reshape(-1), b.reshape(-1)):
                s = s + x * y
            return s
        if name == "size":
            return int(vals[0].size)
        if name == "sum":
            s = F32(0)
            for x in _to_real(vals[0]).reshape(-1, order="F"):
                s = s + x
            return s
        raise NameError(f"intrinsic {name} not supported")


class _MeshIndex(tuple):
    """np.ix_ mesh that squeezes dimensions indexed by a scalar."""

    def __new__(cls, mesh, keep):
        obj = tuple.__new__(cls, mesh)
        obj.keep = keep
        return obj


class Program:
    """All subroutines of a set of Fortran source files."""

    def __init__(self, paths, globals_=None, overrides=None, mpi_stub=False, natives=None):
        self.units = {}
        for p in paths:
            with open(p, encoding="latin-1") as f:
                self.units.update(parse_units(f.read()))
        self.interp = Interp(self.units, globals_, overrides, natives)
        self.interp.mpi_stub = mpi_stub

    def call(self, name, *actuals):
        return self.interp.call(name, list(actuals))


def run_snippet(path, first, last, env, globals_=None, program=None):
    """Execute source lines first..last (1-based, inclusive) of a file as a
    statement sequence in an environment of Var objects; CALLs go to the
    procedures of `program` (a Program) when given."""
    with open(path, encoding="latin-1") as f:
        text = f.read()
    lines = text.split("\n")[first - 1:last]
    stmts = [parse_stmt(no, s) for no, s in logical_lines("\n".join(lines))]
    body = build_blocks([x for x in stmts if x[0] != "decl"])
    unit = Unit("snippet", f"{path}:{first}-{last}", [], body, [])
    interp = Interp(program.units if program is not None else {}, globals_)
    if program is not None:
        interp.natives = program.interp.natives
    ctx = {"unit": unit, "env": env}
    interp.run(ctx, body)
    return env
