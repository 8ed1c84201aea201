"""TEST INFRASTRUCTURE ONLY: a translator from the fixed-form Fortran 77 subset that
compact3d.f is written in to C, so that the reference's own routines can be compiled with
gcc and run beside the oracle restatement (no Fortran compiler exists on either machine).

The translation is mechanical and keeps the reference's semantics as an ``-r8`` build
(``REAL`` and real constants are 8 bytes, ``INTEGER`` 4 bytes, ``COMPLEX`` 16 bytes):

* every routine becomes ``void f77_NAME(...)`` taking every argument by address;
* COMMON blocks are byte arrays (size = the largest declaration seen); each routine
  views its own declaration of a block at its own offsets (storage association);
* arrays keep their declared bounds and column-major order;
* local variables are static and zero-initialised;
* DO loops use the Fortran trip count; labelled DO loops sharing one terminal
  statement close together after it; ``GO TO`` becomes ``goto``;
* ``**`` with an integer exponent is computed by repeated multiplication, otherwise by
  ``pow``; intrinsic generics follow their argument types;
* I/O statements (OPEN, CLOSE, WRITE, READ, PRINT, FORMAT, REWIND) are dropped: they
  only write the reference's .plt files;
* routines that are not requested, and external library routines (FFTW's legacy
  Fortran interface), are called through C functions the caller links in.

Usage: ``python f77c.py SOURCE OUT.c M1 M2 M3 ROOT [ROOT ...]``; writes OUT.c and
OUT.json (the layout of every COMMON block, for the ctypes wrapper).  Nothing produced by
this script is committed: its outputs go to ``oracle/_ref/``.
"""
from __future__ import annotations

import json
import os
import re
import sys

# ----------------------------------------------------------------------------------
# source reading
# ----------------------------------------------------------------------------------


def strip_comment(s: str) -> str:
    out, q = [], None
    for ch in s:
        if q:
            out.append(ch)
            if ch == q:
                q = None
        elif ch in "'\"":
            q = ch
            out.append(ch)
        elif ch == "!":
            break
        else:
            out.append(ch)
    return "".join(out)


def read_statements(path: str, includes: dict, omp: bool = False):
    """Returns a list of (line number, label, statement text) with continuations joined,
    comments removed and INCLUDE lines expanded from `includes` (name -> text).  With
    `omp`, OpenMP directive lines (!$OMP, continued by !$OMP&) become statements
    '$OMP <directive>'."""
    raw = open(path, encoding="latin-1").read().split("\n")
    return _statements(raw, includes, path, omp)


def _statements(raw, includes, where, omp=False):
    stmts = []
    for n, line in enumerate(raw, 1):
        if not line.strip():
            continue
        if omp and line[:5].upper() == "!$OMP":
            if line[5:6] == "&" and stmts and stmts[-1][2].startswith("$OMP"):
                ln, lab, txt = stmts[-1]
                stmts[-1] = (ln, lab, txt + " " + line[6:].strip())
            else:
                stmts.append((n, None, "$OMP " + line[5:].strip()))
            continue
        if line[0] in "cC*!":
            continue
        if line.startswith("\t"):
            rest = line[1:]
            if rest[:1].isdigit() and rest[:1] != "0":     # DEC tab-continuation
                line = "     &" + rest[1:]
            else:
                line = "      " + rest
        label_f = line[:5]
        cont = line[5:6] if len(line) > 5 else " "
        body = line[6:] if len(line) > 6 else ""
        if "\t" in label_f:      # label then tab
            lab, _, rest = line.partition("\t")
            label_f, cont, body = lab, " ", rest
        if label_f.strip().startswith("!"):
            continue
        body = strip_comment(body)
        if cont not in (" ", "0") and stmts:
            ln, lab, txt = stmts[-1]
            stmts[-1] = (ln, lab, txt + body.strip() if txt.endswith(("(", ",")) else txt + " " + body.strip())
            continue
        if not body.strip() and not label_f.strip():
            continue
        m = re.match(r"(?i)^\s*include\s+'([^']+)'", body)
        if m:
            name = m.group(1)
            # an include file outside the source tree (omp_lib.h) declares only the
            # OpenMP runtime's interfaces, which the translation does not use
            stmts.extend(_statements(includes.get(name, "").split("\n"), includes, name, omp))
            continue
        lab = label_f.strip()
        stmts.append((n, int(lab) if lab.isdigit() else None, body.strip()))
    # ';' separates statements on one line (outside character constants)
    out = []
    for n, lab, txt in stmts:
        parts, cur, q = [], [], None
        for ch in txt:
            if q:
                cur.append(ch)
                if ch == q:
                    q = None
            elif ch in "'\"":
                q = ch
                cur.append(ch)
            elif ch == ";":
                parts.append("".join(cur))
                cur = []
            else:
                cur.append(ch)
        parts.append("".join(cur))
        parts = [p.strip() for p in parts if p.strip()]
        for i, p in enumerate(parts):
            out.append((n, lab if i == 0 else None, p))
    return out


# ----------------------------------------------------------------------------------
# expressions
# ----------------------------------------------------------------------------------
DOTOPS = ("EQ", "NE", "LT", "LE", "GT", "GE", "AND", "OR", "NOT", "EQV", "NEQV", "TRUE", "FALSE")
TOK = re.compile(r"""
  (?P<ws>\s+)
 |(?P<str>'(?:[^']|'')*')
 |(?P<num>(?:\d+\.\d*|\.\d+|\d+)(?:[EeDd][+-]?\d+)?)
 |(?P<dot>\.(?:EQ|NE|LT|LE|GT|GE|AND|OR|NOT|EQV|NEQV|TRUE|FALSE)\.)
 |(?P<name>[A-Za-z_]\w*)
 |(?P<op>\*\*|//|==|/=|<=|>=|[-+*/(),:<>=])
""", re.X | re.I)


def tokenize(s: str):
    toks, i = [], 0
    while i < len(s):
        # an integer followed by a dot operator: "1.EQ.2" is 1 .EQ. 2
        m = re.match(r"(\d+)\.(" + "|".join(DOTOPS) + r")\.", s[i:], re.I)
        if m:
            toks.append(("num", m.group(1)))
            i += len(m.group(1))
            continue
        m = TOK.match(s, i)
        if not m:
            raise SyntaxError(f"cannot tokenize {s[i:]!r} in {s!r}")
        i = m.end()
        k = m.lastgroup
        if k == "ws":
            continue
        v = m.group(k)
        if k == "dot":
            v = v.upper()
        if k == "name":
            v = v.upper()
        toks.append((k, v))
    return toks


class P:
    """Recursive-descent parser producing tuples:
    ('num', text, type) ('str', text) ('name', NAME) ('call', NAME, [args])
    ('un', op, e) ('bin', op, a, b) ('log', value)"""

    def __init__(self, toks):
        self.t = toks
        self.i = 0

    def peek(self, k=0):
        j = self.i + k
        return self.t[j] if j < len(self.t) else (None, None)

    def take(self, v=None):
        tok = self.peek()
        if v is not None and tok[1] != v:
            raise SyntaxError(f"expected {v}, got {tok} in {self.t}")
        self.i += 1
        return tok

    def done(self):
        return self.i >= len(self.t)

    def expr(self):
        return self.eqv()

    def eqv(self):
        a = self.lor()
        while self.peek()[1] in (".EQV.", ".NEQV."):
            op = self.take()[1]
            a = ("bin", op, a, self.lor())
        return a

    def lor(self):
        a = self.land()
        while self.peek()[1] == ".OR.":
            self.take()
            a = ("bin", ".OR.", a, self.land())
        return a

    def land(self):
        a = self.lnot()
        while self.peek()[1] == ".AND.":
            self.take()
            a = ("bin", ".AND.", a, self.lnot())
        return a

    def lnot(self):
        if self.peek()[1] == ".NOT.":
            self.take()
            return ("un", ".NOT.", self.lnot())
        return self.rel()

    REL = {".EQ.": "==", ".NE.": "!=", ".LT.": "<", ".LE.": "<=", ".GT.": ">", ".GE.": ">=",
           "==": "==", "/=": "!=", "<": "<", "<=": "<=", ">": ">", ">=": ">="}

    def rel(self):
        a = self.add()
        if self.peek()[1] in self.REL:
            op = self.REL[self.take()[1]]
            a = ("bin", op, a, self.add())
        return a

    def add(self):
        if self.peek()[1] in ("+", "-"):
            op = self.take()[1]
            a = self.mul()
            a = ("un", op, a)
        else:
            a = self.mul()
        while self.peek()[1] in ("+", "-"):
            op = self.take()[1]
            a = ("bin", op, a, self.mul())
        return a

    def mul(self):
        a = self.pow_()
        while self.peek()[1] in ("*", "/"):
            op = self.take()[1]
            a = ("bin", op, a, self.pow_())
        return a

    def pow_(self):
        a = self.prim()
        if self.peek()[1] == "**":
            self.take()
            if self.peek()[1] in ("+", "-"):      # x**-2
                op = self.take()[1]
                b = ("un", op, self.pow_())
            else:
                b = self.pow_()
            return ("bin", "**", a, b)
        return a

    def prim(self):
        k, v = self.peek()
        if k == "num":
            self.take()
            isreal = ("." in v) or re.search(r"[EeDd]", v) is not None
            return ("num", v, "R" if isreal else "I")
        if k == "str":
            self.take()
            return ("str", v)
        if k == "dot" and v in (".TRUE.", ".FALSE."):
            self.take()
            return ("log", v == ".TRUE.")
        if v == "(":
            self.take()
            a = self.expr()
            if self.peek()[1] == ",":      # complex constant (a, b)
                self.take()
                b = self.expr()
                self.take(")")
                return ("call", "CMPLX", [a, b])
            self.take(")")
            return ("par", a)
        if k == "name":
            self.take()
            if self.peek()[1] == "(":
                self.take()
                args = []
                if self.peek()[1] != ")":
                    while True:
                        if self.peek()[1] == ":":
                            raise SyntaxError("array sections are not supported")
                        args.append(self.expr())
                        if self.peek()[1] == ",":
                            self.take()
                            continue
                        break
                self.take(")")
                return ("call", v, args)
            return ("name", v)
        raise SyntaxError(f"unexpected {k} {v} in {self.t}")


def parse_expr(s: str):
    p = P(tokenize(s))
    e = p.expr()
    if not p.done():
        raise SyntaxError(f"trailing tokens in {s!r}: {p.t[p.i:]}")
    return e


# ----------------------------------------------------------------------------------
# declarations
# ----------------------------------------------------------------------------------
CTYPE = {"R": "double", "I": "int", "I8": "long long", "C": "double _Complex", "L": "int", "F": "float",
         "CH": "char"}
SIZE = {"R": 8, "I": 4, "I8": 8, "C": 16, "L": 4, "F": 4}
KEYWORDS = {"DO", "IF", "THEN", "ELSE", "ELSEIF", "ENDIF", "END", "ENDDO", "WHILE", "GO", "GOTO", "TO", "CALL",
            "RETURN", "CONTINUE", "STOP", "EXIT", "CYCLE"}
# OpenMP form: local arrays up to this size are automatic (one per call, so per thread
# inside parallel loops, as a recursive Fortran build has them); larger ones stay static
OMP_AUTO_BYTES = 8 * 1024 * 1024
# static arrays larger than this, and every COMMON block, are heap memory set up when the
# library loads
HEAP_BYTES = 1024 * 1024


def split_top(s: str, sep=","):
    out, depth, cur, q = [], 0, [], None
    for ch in s:
        if q:
            cur.append(ch)
            if ch == q:
                q = None
            continue
        if ch in "'\"":
            q = ch
        if ch == "(":
            depth += 1
        elif ch == ")":
            depth -= 1
        if ch == sep and depth == 0:
            out.append("".join(cur))
            cur = []
        else:
            cur.append(ch)
    out.append("".join(cur))
    return [x.strip() for x in out if x.strip()]


class Var:
    def __init__(self, name, typ=None):
        self.name = name
        self.typ = typ          # 'R','I','I8','C','L','F','CH'
        self.dims = None        # list of (lo_expr, hi_expr) (hi '*' for assumed size)
        self.dummy = False
        self.common = None      # block name
        self.offset = None      # bytes within the block
        self.param = None       # value expression of a PARAMETER
        self.charlen = 0
        self.external = False


class Unit:
    def __init__(self, kind, name, args, rtype=None):
        self.kind = kind
        self.name = name
        self.args = args
        self.rtype = rtype
        self.vars: dict[str, Var] = {}
        self.commons: dict[str, list[str]] = {}
        self.body = []          # (line, label, text)
        self.implicit_none = False

    def var(self, name) -> Var:
        if name not in self.vars:
            self.vars[name] = Var(name)
        return self.vars[name]

    def typeof(self, name) -> str:
        v = self.vars.get(name)
        if v is not None and v.typ:
            return v.typ
        return "I" if name[0] in "IJKLMN" else "R"


TYPE_RE = re.compile(r"(?i)^(real\*8|real\*4|real|double\s+precision|integer\*8|integer\*4|integer|"
                     r"complex\*16|double\s+complex|complex|logical|character\*\(?\s*\d+\s*\)?|character)\b\s*(.*)$")


def type_code(t: str) -> str:
    t = re.sub(r"\s+", " ", t.upper())
    if t in ("REAL", "REAL*8", "DOUBLE PRECISION"):
        return "R"
    if t == "REAL*4":
        return "F"
    if t in ("INTEGER", "INTEGER*4"):
        return "I"
    if t == "INTEGER*8":
        return "I8"
    if t in ("COMPLEX", "COMPLEX*16", "DOUBLE COMPLEX"):
        return "C"
    if t == "LOGICAL":
        return "L"
    if t.startswith("CHARACTER"):
        return "CH"
    raise ValueError(t)


def parse_decl_item(u: Unit, item: str, typ=None, charlen=0):
    m = re.match(r"(?i)^(\w+)\s*(?:\*\s*(\d+))?\s*(?:\((.*)\))?\s*$", item)
    if not m:
        raise SyntaxError(f"declaration {item!r}")
    name = m.group(1).upper()
    v = u.var(name)
    if typ:
        v.typ = typ
        if m.group(2):
            v.charlen = int(m.group(2))
        elif typ == "CH":
            v.charlen = charlen or 1
    if m.group(3):
        dims = []
        for d in split_top(m.group(3)):
            if ":" in d:
                lo, hi = d.split(":", 1)
            else:
                lo, hi = "1", d
            dims.append((lo.strip(), hi.strip()))
        v.dims = dims
    return v


class Program:
    def __init__(self, stmts):
        self.units: dict[str, Unit] = {}
        cur = None
        for ln, lab, txt in stmts:
            up = txt.upper()
            m = re.match(r"^(?:(REAL|INTEGER|DOUBLE\s+PRECISION)\s+)?(SUBROUTINE|FUNCTION|PROGRAM)\s+(\w+)\s*(?:\((.*)\))?\s*$",
                         up)
            if m and cur is None:
                rt = type_code(m.group(1)) if m.group(1) else None
                args = [a.strip() for a in (m.group(4) or "").split(",") if a.strip()]
                cur = Unit(m.group(2), m.group(3), args, rt)
                self.units[cur.name] = cur
                continue
            if cur is not None and re.match(r"^END\s*(SUBROUTINE|FUNCTION|PROGRAM)?\s*\w*$", up) and \
                    not re.match(r"^END\s*(IF|DO)\b", up) and up.replace(" ", "") not in ("ENDDO", "ENDIF"):
                cur = None
                continue
            if cur is not None:
                cur.body.append((ln, lab, txt))


# ----------------------------------------------------------------------------------
# translation of one unit
# ----------------------------------------------------------------------------------
INTRINSIC_REAL1 = {"SQRT": "sqrt", "DSQRT": "sqrt", "EXP": "exp", "DEXP": "exp", "LOG": "log", "ALOG": "log",
                   "DLOG": "log", "LOG10": "log10", "ALOG10": "log10", "SIN": "sin", "DSIN": "sin", "COS": "cos",
                   "DCOS": "cos", "TAN": "tan", "TANH": "tanh", "DTANH": "tanh", "ATAN": "atan", "DATAN": "atan",
                   "ASIN": "asin", "ACOS": "acos", "SINH": "sinh", "COSH": "cosh", "DACOS": "acos", "DASIN": "asin"}


class Translator:
    def __init__(self, prog: Program, params: dict, wanted: set, commons_size: dict, omp: bool = False):
        self.omp = omp
        self.pending_omp = None
        self.redmap = {}
        self.prog = prog
        self.params = params
        self.wanted = wanted
        self.csize = commons_size
        self.externals = set()
        self.ext_funcs = {}
        self.heap = []   # (global name, C type, elements) of the static arrays kept on the heap

    # ---- declarations pass ----
    def declare(self, u: Unit):
        exe = []
        for ln, lab, txt in u.body:
            up = txt.upper().strip()
            if re.match(r"^IMPLICIT\s+NONE", up):
                u.implicit_none = True
                continue
            if up.startswith("IMPLICIT"):
                raise SyntaxError(f"{u.name}:{ln}: IMPLICIT other than NONE is not supported")
            m = re.match(r"^PARAMETER\s*\((.*)\)\s*$", up)
            if m:
                for it in split_top(m.group(1)):
                    nm, ex = it.split("=", 1)
                    v = u.var(nm.strip())
                    v.param = parse_expr(ex)
                continue
            m = re.match(r"^COMMON\s*/\s*(\w+)\s*/\s*(.*)$", up)
            if m:
                blk = m.group(1)
                items = split_top(m.group(2))
                names = []
                for it in items:
                    v = parse_decl_item(u, it)
                    v.common = blk
                    names.append(v.name)
                u.commons.setdefault(blk, []).extend(names)
                continue
            m = re.match(r"^DIMENSION\s+(.*)$", up)
            if m:
                for it in split_top(m.group(1)):
                    parse_decl_item(u, it)
                continue
            m = TYPE_RE.match(txt.strip())
            if m and not re.match(r"(?i)^(real|integer|complex)\s*\(", txt.strip()) and \
                    not re.match(r"(?i)^\w+\s*=", txt.strip()) and not re.match(r"(?i)^(real|integer|double precision|complex)\s+function", txt.strip()):
                tc = type_code(re.sub(r"\*\(?\s*\d+\s*\)?", lambda x: x.group(0) if not x.group(0).startswith("*(") else "*" + re.sub(r"\D", "", x.group(0)), m.group(1)))
                charlen = 0
                if tc == "CH":
                    mm = re.search(r"\d+", m.group(1))
                    charlen = int(mm.group(0)) if mm else 1
                rest = m.group(2).strip()
                if rest.startswith("::"):
                    rest = rest[2:]
                for it in split_top(rest):
                    parse_decl_item(u, it, tc, charlen)
                continue
            if re.match(r"^(EXTERNAL|SAVE|INTRINSIC)\b", up):
                if up.startswith("EXTERNAL"):
                    for it in split_top(up[8:]):
                        u.var(it).external = True
                continue
            if re.match(r"^DATA\b", up):
                raise SyntaxError(f"{u.name}:{ln}: DATA is not supported")
            if re.match(r"^EQUIVALENCE\b", up):
                raise SyntaxError(f"{u.name}:{ln}: EQUIVALENCE is not supported")
            exe.append((ln, lab, txt))
        u.exe = exe
        for a in u.args:
            u.var(a).dummy = True
        # COMMON offsets
        for blk, names in u.commons.items():
            off = 0
            for nm in names:
                v = u.vars[nm]
                v.offset = off
                off += self.nbytes(u, v)
            self.csize[blk] = max(self.csize.get(blk, 0), off)

    def const(self, u: Unit, e):
        """Value of a constant integer (or real) expression."""
        k = e[0]
        if k == "num":
            t = e[1].upper().replace("D", "E")
            return float(t) if e[2] == "R" else int(t)
        if k == "par":
            return self.const(u, e[1])
        if k == "name":
            v = u.vars.get(e[1])
            if v is not None and v.param is not None:
                return self.const(u, v.param)
            if e[1] in self.params:
                return self.params[e[1]]
            raise ValueError(f"{u.name}: {e[1]} is not a constant")
        if k == "un":
            x = self.const(u, e[2])
            return -x if e[1] == "-" else x
        if k == "bin":
            a, b = self.const(u, e[2]), self.const(u, e[3])
            op = e[1]
            if op == "+":
                return a + b
            if op == "-":
                return a - b
            if op == "*":
                return a * b
            if op == "/":
                if isinstance(a, int) and isinstance(b, int):
                    q = abs(a) // abs(b)
                    return q if (a >= 0) == (b >= 0) else -q
                return a / b
            if op == "**":
                return a ** b
        raise ValueError(f"{u.name}: not a constant expression {e}")

    def nbytes(self, u: Unit, v: Var) -> int:
        t = v.typ or u.typeof(v.name)
        sz = v.charlen if t == "CH" else SIZE[t]
        if v.dims:
            for lo, hi in v.dims:
                sz *= self.const(u, parse_expr(hi)) - self.const(u, parse_expr(lo)) + 1
        return sz

    # ---- expression emission: returns (c_text, type) ----
    def ex(self, u: Unit, e):
        k = e[0]
        if k == "num":
            if e[2] == "R":
                t = e[1].upper().replace("D", "E")
                if t.startswith("."):
                    t = "0" + t
                if "." not in t:
                    m = re.match(r"(\d+)(E.*)", t)
                    t = m.group(1) + ".0" + m.group(2)
                elif t.endswith("."):
                    t = t + "0"
                t = t.replace(".E", ".0E")
                return t, "R"
            return str(int(e[1])), "I"
        if k == "log":
            return ("1" if e[1] else "0"), "L"
        if k == "str":
            return "0 /* string */", "CH"
        if k == "par":
            c, t = self.ex(u, e[1])
            return f"({c})", t
        if k == "name":
            return self.ref(u, e[1])
        if k == "un":
            c, t = self.ex(u, e[2])
            if e[1] == ".NOT.":
                return f"(!{c})", "L"
            return f"({e[1]}{c})", t
        if k == "bin":
            op = e[1]
            a, ta = self.ex(u, e[2])
            b, tb = self.ex(u, e[3])
            if op in (".AND.", ".OR."):
                return f"({a} {'&&' if op == '.AND.' else '||'} {b})", "L"
            if op in (".EQV.", ".NEQV."):
                return f"((!!{a}) {'==' if op == '.EQV.' else '!='} (!!{b}))", "L"
            if op in ("==", "!=", "<", "<=", ">", ">="):
                return f"({a} {op} {b})", "L"
            t = self.promote(ta, tb)
            if op == "**":
                if tb in ("I", "I8"):
                    if ta in ("I", "I8"):
                        return f"f77_ipow({a}, {b})", "I"
                    if ta == "C":
                        return f"cpow({a}, (double)({b}))", "C"
                    # integer exponent: repeated multiplication, as compilers expand it
                    return f"f77_powi({a}, {b})", "R"
                if t == "C":
                    return f"cpow({a}, {b})", "C"
                if e[3][0] == "num" and float(e[3][1].upper().replace("D", "E")) == 2.0:
                    return f"f77_powi({a}, 2)", "R"    # compilers fold x**2.0 to x*x
                return f"pow({a}, {b})", "R"
            return f"({a} {op} {b})", t
        if k == "call":
            return self.call_expr(u, e[1], e[2])
        raise ValueError(e)

    @staticmethod
    def promote(ta, tb):
        order = {"L": 0, "I": 1, "I8": 2, "F": 3, "R": 4, "C": 5}
        return ta if order.get(ta, 4) >= order.get(tb, 4) else tb

    def ref(self, u: Unit, name):
        if name in self.redmap:
            return self.redmap[name]
        v = u.vars.get(name)
        if v is not None and v.param is not None:
            val = self.const(u, v.param)
            t = v.typ or u.typeof(name)
            if t in ("R", "F"):
                return repr(float(val)), "R"
            if t == "C":
                return repr(complex(val)), "C"
            return str(int(val)), t
        if name in self.params and (v is None or (v.common is None and not v.dummy and v.dims is None)):
            return str(self.params[name]), "I"
        t = u.typeof(name)
        if v is None and not (u.kind == "FUNCTION" and name == u.name):
            v = u.var(name)              # an implicitly typed local scalar
        if v is not None and v.dims:
            return f"v_{name}", t        # whole array (pointer)
        if v is not None and (v.dummy or v.common):
            return f"(*v_{name})", t
        if u.kind == "FUNCTION" and name == u.name:
            return "f77_result", u.rtype or u.typeof(name)
        return f"v_{name}", t

    def index(self, u: Unit, v: Var, args):
        """Linear index of an array element (0-based) in column-major order."""
        terms = []
        stride = "1"
        for n, (a, (lo, hi)) in enumerate(zip(args, v.dims)):
            ca, _ = self.ex(u, a)
            clo, _ = self.ex(u, parse_expr(lo))
            terms.append(f"(({ca}) - ({clo}))" + ("" if stride == "1" else f" * ({stride})"))
            if n < len(v.dims) - 1:
                chi, _ = self.ex(u, parse_expr(hi))
                ext = f"(({chi}) - ({clo}) + 1)"
                stride = ext if stride == "1" else f"{stride} * {ext}"
        return " + ".join(terms)

    def call_expr(self, u: Unit, name, args):
        v = u.vars.get(name)
        if v is not None and v.dims:           # array element
            t = v.typ or u.typeof(name)
            return f"v_{name}[{self.index(u, v, args)}]", t
        cargs = [self.ex(u, a) for a in args]
        ts = [t for _, t in cargs]
        cs = [c for c, _ in cargs]
        if name in INTRINSIC_REAL1:
            if ts and ts[0] == "C":
                return f"c{INTRINSIC_REAL1[name]}({cs[0]})", "C"
            return f"{INTRINSIC_REAL1[name]}((double)({cs[0]}))", "R"
        if name in ("ABS", "DABS", "IABS", "CABS"):
            if ts[0] == "C":
                return f"cabs({cs[0]})", "R"
            if ts[0] in ("I", "I8"):
                return f"abs({cs[0]})", "I"
            return f"fabs({cs[0]})", "R"
        if name in ("MAX", "MIN", "AMAX1", "AMIN1", "DMAX1", "DMIN1", "MAX0", "MIN0", "AMAX0", "AMIN0", "MAX1", "MIN1"):
            ismax = "MAX" in name
            allint = all(t in ("I", "I8") for t in ts) and name not in ("AMAX1", "AMIN1", "DMAX1", "DMIN1", "AMAX0", "AMIN0")
            f = ("f77_imax" if ismax else "f77_imin") if allint else ("f77_dmax" if ismax else "f77_dmin")
            acc = cs[0]
            for c in cs[1:]:
                acc = f"{f}({acc}, {c})"
            rt = "I" if allint else "R"
            if name in ("MAX1", "MIN1"):
                return f"((int)({acc}))", "I"
            return acc, rt
        if name == "MOD" or name == "AMOD" or name == "DMOD":
            if all(t in ("I", "I8") for t in ts):
                return f"(({cs[0]}) % ({cs[1]}))", "I"
            return f"fmod({cs[0]}, {cs[1]})", "R"
        if name in ("SIGN", "DSIGN", "ISIGN"):
            if all(t in ("I", "I8") for t in ts):
                return f"f77_isign({cs[0]}, {cs[1]})", "I"
            return f"f77_sign({cs[0]}, {cs[1]})", "R"
        if name in ("FLOAT", "DBLE", "DFLOAT", "SNGL"):
            return f"((double)({cs[0]}))", "R"
        if name in ("REAL", "DREAL"):
            if ts[0] == "C":
                return f"creal({cs[0]})", "R"
            return f"((double)({cs[0]}))", "R"
        if name in ("AIMAG", "DIMAG"):
            return f"cimag({cs[0]})", "R"
        if name in ("CONJG", "DCONJG"):
            return f"conj({cs[0]})", "C"
        if name in ("CMPLX", "DCMPLX"):
            im = cs[1] if len(cs) > 1 else "0.0"
            return f"f77_cmplx({cs[0]}, {im})", "C"
        if name in ("INT", "IFIX", "IDINT"):
            return f"((int)({cs[0]}))", "I"
        if name in ("NINT", "IDNINT"):
            return f"((int)lround({cs[0]}))", "I"
        if name in ("ANINT", "DNINT"):
            return f"round({cs[0]})", "R"
        if name in ("AINT", "DINT"):
            return f"trunc({cs[0]})", "R"
        if name in ("ATAN2", "DATAN2"):
            return f"atan2({cs[0]}, {cs[1]})", "R"
        if name == "SQRT":
            return f"sqrt({cs[0]})", "R"
        # a FUNCTION subprogram or an external function: called by reference
        rt = u.typeof(name)
        fu = self.prog.units.get(name)
        if fu is not None and fu.kind == "FUNCTION":
            rt = fu.rtype or rt
        if name not in self.wanted:
            self.ext_funcs[name] = rt
        argl = ", ".join(self.actual(u, a) for a in args)
        return f"f77_{name}({argl})", rt

    def actual(self, u: Unit, a):
        """An actual argument: the address of a variable, array, array element or a
        temporary holding an expression's value."""
        if a[0] == "name":
            nm = a[1]
            v = u.vars.get(nm)
            if v is not None and v.param is None and (nm not in self.params or v.common or v.dummy or v.dims):
                if v.dims:
                    return f"v_{nm}"
                if v.dummy or v.common:
                    return f"v_{nm}"
                return f"&v_{nm}"
            if v is None and nm not in self.params:
                u.var(nm)
                return f"&v_{nm}"
        if a[0] == "call":
            v = u.vars.get(a[1])
            if v is not None and v.dims:
                return f"&v_{a[1]}[{self.index(u, v, a[2])}]"
        c, t = self.ex(u, a)
        if t == "CH":
            return "(void *)0"
        return f"&({CTYPE.get(t, 'double')}){{{c}}}"

    # ---- statements ----
    def unit_c(self, u: Unit):
        self.declare(u)
        out = []
        params = []
        for a in u.args:
            v = u.vars[a]
            t = v.typ or u.typeof(a)
            params.append(f"{CTYPE[t]} *v_{a}")
        sig = f"void f77_{u.name}({', '.join(params) or 'void'})"
        if u.kind == "FUNCTION":
            rt = u.rtype or u.typeof(u.name)
            sig = f"{CTYPE[rt]} f77_{u.name}({', '.join(params) or 'void'})"
        self.do_stack = []
        self.goto_targets = set()
        for ln, lab, txt in u.exe:
            for m in re.finditer(r"(?i)\bGO\s*TO\s*(\d+)", txt):
                self.goto_targets.add(int(m.group(1)))
        if self.omp:
            # every name the routine uses exists before the first parallel loop is emitted,
            # so that its firstprivate clause lists the scalars first used inside the loop
            for ln, lab, txt in u.exe:
                up = txt.upper().strip()
                if up.startswith("$OMP") or re.match(r"^(CALL|WRITE|READ|PRINT|FORMAT|OPEN|CLOSE)\b", up):
                    if not up.startswith("CALL"):
                        continue
                try:
                    toks = tokenize(re.sub(r"^CALL\s+\w+", "", up))
                except SyntaxError:
                    continue
                for i, (k, v) in enumerate(toks):
                    nxt = toks[i + 1][1] if i + 1 < len(toks) else None
                    if k == "name" and nxt != "(" and v not in self.params and v not in KEYWORDS:
                        if v not in u.vars and not (u.kind == "FUNCTION" and v == u.name):
                            u.var(v)
        body = []
        self.ind = 1
        for ln, lab, txt in u.exe:
            try:
                self.stmt(u, ln, lab, txt, body)
            except Exception as exc:
                raise SyntaxError(f"{u.name} line {ln}: {txt!r}: {exc}") from exc
        if self.do_stack:
            raise SyntaxError(f"{u.name}: unclosed DO loops {self.do_stack}")
        out.append(sig + " {")
        if u.kind == "FUNCTION":
            out.append(f"  {CTYPE[u.rtype or u.typeof(u.name)]} f77_result = 0;")
        # locals and common views
        for nm, v in u.vars.items():
            if v.param is not None or v.dummy or v.external:
                continue
            if u.kind == "FUNCTION" and nm == u.name:
                continue
            t = v.typ or u.typeof(nm)
            if t == "CH":
                if v.common:
                    continue
                n = v.charlen * (1 if not v.dims else self.nelems(u, v))
                out.append(f"  static char v_{nm}[{n}];")
                continue
            if v.common:
                out.append(f"  {CTYPE[t]} *v_{nm} = ({CTYPE[t]} *)(f77c_{v.common} + {v.offset});")
            elif v.dims:
                try:
                    ne = self.nelems(u, v)
                    # OpenMP: per-call (per-thread) arrays, except the channel-sized ones
                    auto = self.omp and ne * SIZE.get(t, 8) <= OMP_AUTO_BYTES
                    if not auto and ne * SIZE.get(t, 8) > HEAP_BYTES:
                        # a channel-sized array: zeroed heap memory allocated when the
                        # library loads (static data of this size exceeds what the code
                        # model addresses)
                        gname = f"f77l_{u.name}_{nm}"
                        self.heap.append((gname, CTYPE[t], ne))
                        out.append(f"  {CTYPE[t]} *v_{nm} = {gname};")
                    else:
                        out.append(f"  {'' if auto else 'static '}{CTYPE[t]} v_{nm}[{ne}];")
                except ValueError:
                    # automatic array sized by dummy arguments: a zeroed stack array
                    n = " * ".join(f"(({self.ex(u, parse_expr(hi))[0]}) - ({self.ex(u, parse_expr(lo))[0]}) + 1)"
                                   for lo, hi in v.dims)
                    out.append(f"  {CTYPE[t]} v_{nm}[{n}]; memset(v_{nm}, 0, sizeof(v_{nm}));")
            elif self.used_as_var(u, nm):
                out.append(f"  {CTYPE[t]} v_{nm} = 0;" if self.omp else f"  static {CTYPE[t]} v_{nm};")
        out.extend(body)
        if u.kind == "FUNCTION":
            out.append("  return f77_result;")
        out.append("}")
        return sig, "\n".join(out)

    def nelems(self, u, v):
        n = 1
        for lo, hi in v.dims:
            if hi == "*":
                raise SyntaxError(f"{u.name}: local array {v.name} of assumed size")
            n *= self.const(u, parse_expr(hi)) - self.const(u, parse_expr(lo)) + 1
        return n

    def used_as_var(self, u, nm):
        return True

    def emit(self, body, s):
        body.append("  " * self.ind + s)

    def stmt(self, u: Unit, ln, lab, txt, body):
        up = txt.upper().strip()
        if lab is not None and lab in self.goto_targets:
            self.emit(body, f"L{lab}:;")
        self.simple(u, up, txt, body, lab)
        # close labelled DO loops ending here
        while self.do_stack and self.do_stack[-1][0] is not None and self.do_stack[-1][0] == lab:
            self.close_do(body)

    def simple(self, u, up, txt, body, lab):
        if up.startswith("$OMP"):
            if self.omp:
                self.omp_directive(up[4:].strip())
            return
        if up in ("CONTINUE",):
            return
        if re.match(r"^(OPEN|CLOSE|WRITE|READ|PRINT|FORMAT|REWIND|BACKSPACE|INQUIRE|FLUSH)\b", up) or \
                re.match(r"^(OPEN|CLOSE|WRITE|READ|PRINT|FORMAT)\s*\(", up):
            return
        if re.match(r"^RETURN$", up):
            self.emit(body, "return" + (" f77_result;" if u.kind == "FUNCTION" else ";"))
            return
        if re.match(r"^STOP\b", up):
            self.emit(body, "f77_stop();")
            return
        m = re.match(r"^GO\s*TO\s*(\d+)$", up)
        if m:
            self.emit(body, f"goto L{m.group(1)};")
            return
        if up in ("EXIT",):
            self.emit(body, "break;")
            return
        if up in ("CYCLE",):
            self.emit(body, "continue;")
            return
        m = re.match(r"^DO\s+WHILE\s*\((.*)\)$", up)
        if m:
            c, _ = self.ex(u, parse_expr(m.group(1)))
            self.emit(body, f"{{ while ({c}) {{")
            self.do_stack.append((None, "while"))
            self.ind += 1
            return
        m = re.match(r"^DO\s*(\d+)?\s*,?\s*(\w+)\s*=\s*(.*)$", up)
        if m and not re.match(r"^DO\w*\s*=", up):
            lab_end = int(m.group(1)) if m.group(1) else None
            var = m.group(2)
            parts = split_top(m.group(3))
            s, e = self.ex(u, parse_expr(parts[0]))[0], self.ex(u, parse_expr(parts[1]))[0]
            st = self.ex(u, parse_expr(parts[2]))[0] if len(parts) > 2 else "1"
            vt = u.typeof(var)
            vref = self.ref(u, var)[0]
            d = len(self.do_stack)
            ct = CTYPE[vt]
            if self.pending_omp is not None:
                if any(u.vars.get(nm) is not None and u.vars[nm].dims for _, nm in self.pending_omp["red"]):
                    self.pending_omp = None   # an array reduction (WALLSS's WSM): the loop runs on one thread
                else:
                    self.parallel_do(u, body, lab_end, vref, ct, s, e, st, d)
                    return
            self.emit(body, f"{{ {ct} s{d} = {st}; long n{d} = (long)((({e}) - ({s}) + s{d}) / s{d}); "
                            f"for ({vref} = {s}; n{d} > 0; --n{d}, {vref} += s{d}) {{")
            self.do_stack.append((lab_end, "do"))
            self.ind += 1
            return
        if up in ("ENDDO", "END DO"):
            if not self.do_stack or self.do_stack[-1][0] is not None:
                raise SyntaxError("ENDDO without DO")
            self.close_do(body)
            return
        m = re.match(r"^IF\s*\((.*)$", up)
        if m:
            cond, rest = self.split_paren(txt.strip()[2:].strip())
            c, _ = self.ex(u, parse_expr(cond))
            r = rest.strip()
            if r.upper() == "THEN":
                self.emit(body, f"if ({c}) {{")
                self.ind += 1
                return
            if re.match(r"^\d+\s*,\s*\d+\s*,\s*\d+$", r):
                raise SyntaxError("arithmetic IF")
            self.emit(body, f"if ({c}) {{")
            self.ind += 1
            self.simple(u, r.upper(), r, body, None)
            self.ind -= 1
            self.emit(body, "}")
            return
        m = re.match(r"^ELSE\s*IF\s*\((.*)\)\s*THEN$", up)
        if m:
            cond, _ = self.split_paren(re.sub(r"(?i)^ELSE\s*IF", "", txt.strip()).strip())
            c, _ = self.ex(u, parse_expr(cond))
            self.ind -= 1
            self.emit(body, f"}} else if ({c}) {{")
            self.ind += 1
            return
        if up == "ELSE":
            self.ind -= 1
            self.emit(body, "} else {")
            self.ind += 1
            return
        if up in ("ENDIF", "END IF"):
            self.ind -= 1
            self.emit(body, "}")
            return
        m = re.match(r"^CALL\s+(\w+)\s*(?:\((.*)\))?\s*$", up)
        if m:
            name = m.group(1)
            args = [parse_expr(a) for a in split_top(txt.strip()[txt.upper().index("CALL") + 4:].strip()[len(name):].strip()[1:-1])] \
                if m.group(2) is not None else []
            if name not in self.wanted:
                self.externals.add(name)
            self.emit(body, f"f77_{name}({', '.join(self.actual(u, a) for a in args)});")
            return
        # assignment
        lhs, eq, rhs = self.split_assign(txt.strip())
        if eq:
            le = parse_expr(lhs)
            c, t = self.ex(u, parse_expr(rhs))
            lc, lt = self.ex(u, le)
            if lt in ("I", "I8") and t in ("R", "F", "C"):
                c = f"({CTYPE[lt]})({'creal(' + c + ')' if t == 'C' else c})"
            elif lt in ("R", "F") and t == "C":
                c = f"creal({c})"
            self.emit(body, f"{lc} = {c};")
            return
        raise SyntaxError(f"unsupported statement {txt!r}")

    def close_do(self, body):
        ent = self.do_stack.pop()
        self.ind -= 1
        if ent[1] == "omp":
            self.emit(body, "}")
            for line in ent[2]:
                self.emit(body, line)
            self.emit(body, "}")
            self.redmap = {}
        else:
            self.emit(body, "}}")

    def omp_directive(self, text: str):
        """!$OMP PARALLEL DO [PRIVATE(list)] [REDUCTION(op:list)]: applies to the next DO."""
        t = text.upper()
        if not re.match(r"^PARALLEL\s+DO\b", t):
            raise SyntaxError(f"unsupported OpenMP directive {text!r}")
        priv = []
        for m in re.finditer(r"PRIVATE\s*\(([^)]*)\)", t):
            priv += [x.strip() for x in m.group(1).split(",") if x.strip()]
        red = []
        for m in re.finditer(r"REDUCTION\s*\(\s*([+*]|MAX|MIN)\s*:([^)]*)\)", t):
            red += [(m.group(1), x.strip()) for x in m.group(2).split(",") if x.strip()]
        self.pending_omp = dict(private=priv, red=red)

    def parallel_do(self, u, body, lab_end, vref, ct, s, e, st, d):
        """A Fortran PARALLEL DO as an OpenMP loop over the trip count.  Every local scalar is
        firstprivate (the loop's own and inner DO variables included, as Fortran makes them
        private, and temporaries the directive may not list); arrays the directive lists are
        private; a reduction variable gets a local accumulator folded into it after the loop."""
        pend, self.pending_omp = self.pending_omp, None
        redn = {nm for _, nm in pend["red"]}
        pre, post = [], []
        for op, nm in pend["red"]:
            t = u.typeof(nm)
            c = CTYPE[t]
            init = {"+": "0", "*": "1", "MAX": "-HUGE_VAL" if t in ("R", "F") else "INT_MIN",
                    "MIN": "HUGE_VAL" if t in ("R", "F") else "INT_MAX"}[op]
            orig = self.ref(u, nm)[0]
            pre.append(f"{c} r_{nm} = {init};")
            if op in ("+", "*"):
                post.append(f"{orig} = {orig} {op} r_{nm};")
            else:
                f = ("f77_dmax" if op == "MAX" else "f77_dmin") if t in ("R", "F") else ("f77_imax" if op == "MAX" else "f77_imin")
                post.append(f"{orig} = {f}({orig}, r_{nm});")
        fp, pv = [], []
        for nm, v in u.vars.items():
            if v.param is not None or v.dummy or v.external or v.common or nm in redn:
                continue
            if u.kind == "FUNCTION" and nm == u.name:
                continue
            t = v.typ or u.typeof(nm)
            if t == "CH":
                continue
            if v.dims:
                if nm in pend["private"]:
                    pv.append(f"v_{nm}")
            else:
                fp.append(f"v_{nm}")
        self.emit(body, f"{{ {ct} s{d} = {st}; {ct} b{d} = {s}; long n{d} = (long)((({e}) - (b{d}) + s{d}) / s{d});")
        for line in pre:
            self.emit(body, line)
        clauses = []
        if fp:
            clauses.append("firstprivate(" + ", ".join(fp) + ")")
        if pv:
            clauses.append("private(" + ", ".join(pv) + ")")
        for op, nm in pend["red"]:
            clauses.append(f"reduction({'max' if op == 'MAX' else 'min' if op == 'MIN' else op}:r_{nm})")
        self.emit(body, "#pragma omp parallel for schedule(static) " + " ".join(clauses))
        self.emit(body, f"for (long i{d} = 0; i{d} < n{d}; ++i{d}) {{ {vref} = b{d} + ({ct})i{d} * s{d};")
        self.redmap = {nm: (f"r_{nm}", u.typeof(nm)) for _, nm in pend["red"]}
        self.do_stack.append((lab_end, "omp", post))
        self.ind += 1

    @staticmethod
    def split_paren(s: str):
        """'(cond) rest' -> ('cond', 'rest')."""
        assert s.startswith("("), s
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
                if depth == 0:
                    return s[1:i], s[i + 1:]
        raise SyntaxError("unbalanced parentheses")

    @staticmethod
    def split_assign(s: str):
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
            elif ch == "=" and depth == 0 and s[i + 1:i + 2] != "=" and s[i - 1:i] not in ("<", ">", "/", "="):
                return s[:i], "=", s[i + 1:]
        return s, None, None


HEADER = r"""/* Generated from the reference's Fortran source by oracle/f77c.py; not committed. */
#include <math.h>
#include <complex.h>
#include <stdlib.h>
#include <string.h>
#include <limits.h>
static inline int f77_ipow(int a, int b) { int r = 1; if (b < 0) return (a == 1) ? 1 : (a == -1 ? ((b & 1) ? -1 : 1) : 0); while (b--) r *= a; return r; }
static inline double f77_powi(double x, int n) {
    /* x**n for an integer n: binary powering, as compilers expand integer powers */
    if (n < 0) return 1.0 / f77_powi(x, -n);
    double r = 1.0; int first = 1;
    while (n) { if (n & 1) { r = first ? x : r * x; first = 0; } n >>= 1; if (n) x = x * x; }
    return first ? 1.0 : r;
}
static inline int f77_imax(int a, int b) { return a > b ? a : b; }
static inline int f77_imin(int a, int b) { return a < b ? a : b; }
static inline double f77_dmax(double a, double b) { return a > b ? a : b; }
static inline double f77_dmin(double a, double b) { return a < b ? a : b; }
static inline double f77_sign(double a, double b) { return b >= 0 ? fabs(a) : -fabs(a); }
static inline int f77_isign(int a, int b) { return b >= 0 ? abs(a) : -abs(a); }
static inline double _Complex f77_cmplx(double a, double b) { return a + b * _Complex_I; }
int f77_stop_flag;
static void f77_stop(void) { f77_stop_flag = 1; }
"""


def translate(src, out_c, m1, m2, m3, roots, fortran_dir=None, omp=False):
    fortran_dir = fortran_dir or os.path.dirname(src)
    includes = {}
    for name in ("PARAM.H", "COMMON1.FI"):
        includes[name] = open(os.path.join(fortran_dir, name), encoding="latin-1").read()
    includes["PARAM.H"] = f"      PARAMETER (M1={m1},M2={m2},M3={m3})\n"
    prog = Program(read_statements(src, includes, omp))
    # routines reachable from the roots through CALL statements and function references
    wanted, stack = set(), list(roots)
    while stack:
        n = stack.pop()
        if n in wanted or n not in prog.units:
            continue
        wanted.add(n)
        for ln, lab, txt in prog.units[n].body:
            for m in re.finditer(r"(?i)\bCALL\s+(\w+)", txt):
                stack.append(m.group(1).upper())
            for fname, fu in prog.units.items():
                if fu.kind == "FUNCTION" and re.search(r"(?i)\b" + fname + r"\s*\(", txt):
                    stack.append(fname)
    csize = {}
    tr = Translator(prog, {}, wanted, csize, omp)
    sigs, bodies = [], []
    for n in sorted(wanted):
        s, b = tr.unit_c(prog.units[n])
        sigs.append(s + ";")
        bodies.append(b)
    lines = [HEADER]
    for blk, sz in sorted(csize.items()):
        lines.append(f"unsigned char *f77c_{blk};   /* COMMON /{blk}/, {sz} bytes */")
    for x in sorted(tr.externals):
        lines.append(f"void f77_{x}();")
    for x, t in sorted(tr.ext_funcs.items()):
        lines.append(f"{CTYPE[t]} f77_{x}();")
    for gname, ct, ne in tr.heap:
        lines.append(f"static {ct} *{gname};")
    # COMMON blocks and the large static arrays: zeroed memory, allocated once at load time
    lines.append("__attribute__((constructor)) static void f77_load(void) {")
    for blk, sz in sorted(csize.items()):
        lines.append(f"  f77c_{blk} = (unsigned char *)calloc({(sz + 15) // 16 * 16}, 1);")
    for gname, ct, ne in tr.heap:
        lines.append(f"  {gname} = ({ct} *)calloc({ne}, sizeof({ct}));")
    lines.append("}")
    lines.extend(sigs)
    lines.extend(bodies)
    open(out_c, "w").write("\n".join(lines) + "\n")
    # layout of every COMMON block as the first translated routine that names it declares it
    layout = {}
    for n in sorted(wanted):
        u = prog.units[n]
        for blk, names in u.commons.items():
            if blk in layout:
                continue
            ent = []
            for nm in names:
                v = u.vars[nm]
                t = v.typ or u.typeof(nm)
                dims = [[tr.const(u, parse_expr(lo)), tr.const(u, parse_expr(hi))] for lo, hi in v.dims] if v.dims else []
                ent.append(dict(name=nm, type=t, offset=v.offset, dims=dims))
            layout[blk] = dict(size=csize[blk], vars=ent)
    json.dump(dict(layout=layout, routines=sorted(wanted), externals=sorted(tr.externals | set(tr.ext_funcs))),
              open(os.path.splitext(out_c)[0] + ".json", "w"), indent=1)
    return sorted(wanted), sorted(tr.externals | set(tr.ext_funcs))


if __name__ == "__main__":
    a = sys.argv[1:]
    w, ext = translate(a[0], a[1], int(a[2]), int(a[3]), int(a[4]), [x.upper() for x in a[5:]])
    print("translated:", " ".join(w))
    print("external:", " ".join(ext))
