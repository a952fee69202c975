#!/usr/bin/env python3
"""Mechanical Fortran-77 -> C translator used to run the reference's own
kernels as a second, independent oracle.

TEST INFRASTRUCTURE ONLY.  Nothing in the product imports or links this.

The reference library (LSMLIB) keeps all of its level-set arithmetic in
fixed-form Fortran 77, and this image has no Fortran compiler.  The subset
of Fortran the hot-path files use is small and regular (subroutines,
INTEGER / INTEGER*1 / REAL / LOGICAL declarations with explicit bounds,
PARAMETER, DO/ENDDO, block and logical IF, CALL, EXIT, RETURN, and the
intrinsics ABS MAX MIN SQRT SIN COS SIGN MOD), so this script reads the
reference source files where they lie and emits equivalent C99:

* every dummy argument becomes a pointer (Fortran passes by reference);
  the lowercase-name-plus-underscore symbol that gfortran would export is
  kept, so the result links where the Fortran objects would;
* arrays keep their declared lower/upper bounds and column-major layout;
* real literals and REAL variables follow the reference's CMake build:
  ``--precision double`` mimics ``gfortran -fdefault-real-8
  -fdefault-double-8`` (every REAL and every real literal is double),
  ``--precision single`` mimics the USE_SINGLE_PRECISION build (REAL is
  float, ``d``-exponent literals stay double, mixed expressions promote);
* integer powers ``x**n`` become repeated multiplication the way gfortran
  expands them; MAX/MIN follow gfortran's ``a > b ? a : b`` selection;
* the ``@lsmlib_zero_tol@`` / ``@tiny_nonzero_number@`` template values are
  substituted with the values src/CMakeLists.txt:10-20 gives them.

The output is compiled with ``-O2 -ffp-contract=off`` so that no fused
multiply-add changes a rounding the Fortran build (x86-64, SSE2, no FMA)
would not make.

Usage:  f77ref.py --precision double OUT.c SRC.f [SRC.f ...]
"""
import argparse
import re
import sys

TEMPLATES = {
    "double": {"@lsmlib_zero_tol@": "1.e-11", "@tiny_nonzero_number@": "1.d-36"},
    "single": {"@lsmlib_zero_tol@": "1.e-5", "@tiny_nonzero_number@": "1.d-36"},
}

INTRINSICS = {"abs", "max", "min", "sqrt", "sin", "cos", "sign", "mod",
              "dble", "real", "int", "exp", "log", "dabs", "dsqrt", "dmax1",
              "dmin1", "amax1", "amin1", "float"}


class TranslateError(Exception):
    pass


# --------------------------------------------------------------------------
# fixed-form reader
# --------------------------------------------------------------------------
def logical_lines(text, fname):
    """Yield (first_line_number, statement_text) of fixed-form source."""
    stmts = []
    for n, raw in enumerate(text.splitlines(), 1):
        if not raw.strip():
            continue
        if raw[0] in "cC*!":
            continue
        lead = len(raw) - len(raw.lstrip(" "))
        if lead < 6 and raw[lead:lead + 1] == "\t":
            # tab format: a tab in columns 1-6 starts the statement field
            rest = raw[lead + 1:]
            if rest[:1] in "123456789":
                cont, body = True, rest[1:]
            else:
                cont, body = False, rest
        else:
            head = raw[:6].ljust(6)
            if head[:5].strip() and not head[:5].strip().isdigit():
                # not a label: free text in columns 1-5 (never used here)
                raise TranslateError(f"{fname}:{n}: unexpected text in cols 1-5")
            cont = head[5] not in " 0"
            body = raw[6:]
        # strip trailing '!' comments (the files carry no character data)
        if "!" in body:
            body = body[: body.index("!")]
        body = body.replace("\t", " ")
        if cont:
            if not stmts:
                raise TranslateError(f"{fname}:{n}: continuation without statement")
            stmts[-1][1] += " " + body
        else:
            stmts.append([n, body])
    out = []
    for n, s in stmts:
        for part in split_top(s, ";"):
            if part.strip():
                out.append((n, part.strip()))
    return out


def split_top(s, sep):
    """Split on `sep` at parenthesis depth 0."""
    parts, depth, cur = [], 0, []
    for ch in s:
        if ch == "(":
            depth += 1
        elif ch == ")":
            depth -= 1
        if ch == sep and depth == 0:
            parts.append("".join(cur))
            cur = []
        else:
            cur.append(ch)
    parts.append("".join(cur))
    return parts


# --------------------------------------------------------------------------
# expressions
# --------------------------------------------------------------------------
TOKEN_RE = re.compile(r"""
    (?P<ws>\s+)
  | (?P<dotop>\.(?:lt|le|gt|ge|eq|ne|and|or|not|true|false|eqv|neqv)\.)
  | (?P<real>(?:\d+\.\d*|\.\d+|\d+)(?:[eEdD][+-]?\d+)|\d+\.\d*|\.\d+)
  | (?P<int>\d+)
  | (?P<name>[A-Za-z_][A-Za-z_0-9]*)
  | (?P<op>\*\*|<=|>=|==|/=|<|>|[-+*/(),:])
""", re.VERBOSE | re.IGNORECASE)


def tokenize(s):
    toks, pos = [], 0
    while pos < len(s):
        m = TOKEN_RE.match(s, pos)
        if not m:
            raise TranslateError(f"cannot tokenize {s[pos:]!r}")
        pos = m.end()
        kind = m.lastgroup
        if kind == "ws":
            continue
        text = m.group(kind)
        if kind == "dotop":
            text = text.lower()
        if kind == "name":
            text = text.lower()
        toks.append((kind, text))
    return toks


class Parser:
    """Precedence-climbing parser producing tuples:
    ('num', text, kind) ('var', name) ('ref', name, [args]) ('un', op, x)
    ('bin', op, a, b)"""

    def __init__(self, toks):
        self.t = toks
        self.i = 0

    def peek(self):
        return self.t[self.i] if self.i < len(self.t) else (None, None)

    def take(self, text=None):
        tok = self.peek()
        if text is not None and tok[1] != text:
            raise TranslateError(f"expected {text!r}, got {tok!r}")
        self.i += 1
        return tok

    def parse(self):
        e = self.p_eqv()
        if self.i != len(self.t):
            raise TranslateError(f"trailing tokens {self.t[self.i:]}")
        return e

    def p_eqv(self):
        a = self.p_or()
        while self.peek()[1] in (".eqv.", ".neqv."):
            op = "==" if self.take()[1] == ".eqv." else "!="
            a = ("bin", op, ("un", "!!", a), ("un", "!!", self.p_or()))
        return a

    def p_or(self):
        a = self.p_and()
        while self.peek()[1] == ".or.":
            self.take()
            a = ("bin", "||", a, self.p_and())
        return a

    def p_and(self):
        a = self.p_not()
        while self.peek()[1] == ".and.":
            self.take()
            a = ("bin", "&&", a, self.p_not())
        return a

    def p_not(self):
        if self.peek()[1] == ".not.":
            self.take()
            return ("un", "!", self.p_not())
        return self.p_rel()

    REL = {".lt.": "<", ".le.": "<=", ".gt.": ">", ".ge.": ">=", ".eq.": "==",
           ".ne.": "!=", "<": "<", "<=": "<=", ">": ">", ">=": ">=",
           "==": "==", "/=": "!="}

    def p_rel(self):
        a = self.p_add()
        if self.peek()[1] in self.REL:
            op = self.REL[self.take()[1]]
            a = ("bin", op, a, self.p_add())
        return a

    def p_add(self):
        # Fortran: a leading unary +/- applies to the following term
        if self.peek()[1] in ("+", "-"):
            op = self.take()[1]
            a = self.p_mul()
            if op == "-":
                a = ("un", "-", a)
        else:
            a = self.p_mul()
        while self.peek()[1] in ("+", "-"):
            op = self.take()[1]
            a = ("bin", op, a, self.p_mul())
        return a

    def p_mul(self):
        a = self.p_pow()
        while self.peek()[1] in ("*", "/"):
            op = self.take()[1]
            a = ("bin", op, a, self.p_pow())
        return a

    def p_pow(self):
        a = self.p_prim()
        if self.peek()[1] == "**":
            self.take()
            # right associative; exponent may carry a sign
            if self.peek()[1] in ("+", "-"):
                op = self.take()[1]
                b = self.p_pow()
                if op == "-":
                    b = ("un", "-", b)
            else:
                b = self.p_pow()
            a = ("bin", "**", a, b)
        return a

    def p_prim(self):
        kind, text = self.take()
        if kind == "real":
            return ("num", text, "real")
        if kind == "int":
            return ("num", text, "int")
        if kind == "dotop" and text in (".true.", ".false."):
            return ("num", "1" if text == ".true." else "0", "logical")
        if kind == "name":
            if self.peek()[1] == "(":
                self.take("(")
                args = []
                if self.peek()[1] != ")":
                    args.append(self.p_or())
                    while self.peek()[1] == ",":
                        self.take()
                        args.append(self.p_or())
                self.take(")")
                return ("ref", text, args)
            return ("var", text)
        if text == "(":
            e = self.p_or()
            self.take(")")
            return ("paren", e)
        raise TranslateError(f"unexpected token {text!r}")


def parse_expr(s):
    return Parser(tokenize(s)).parse()


# --------------------------------------------------------------------------
# subroutine model
# --------------------------------------------------------------------------
class Var:
    def __init__(self, name, ftype):
        self.name = name
        self.ftype = ftype      # 'real' | 'int' | 'int1' | 'logical'
        self.dims = None        # list of (lo_expr, hi_expr) or None
        self.is_arg = False
        self.is_param = False


class Unit:
    def __init__(self, name, args, src, line):
        self.name = name
        self.args = args
        self.vars = {}
        self.params = []        # (name, expr_text) in source order
        self.body = []          # (line, stmt)
        self.written = set()    # names assigned in this unit
        self.calls = []         # (callee, [actual arg exprs])
        self.src = src
        self.line = line


class Translator:
    def __init__(self, precision):
        self.prec = precision
        self.real_c = "double" if precision == "double" else "float"

    # ---- types -----------------------------------------------------------
    def ctype(self, ftype):
        return {"real": self.real_c, "int": "int", "int1": "signed char",
                "logical": "int", "double": "double"}[ftype]

    def lit_type(self, text):
        if "d" in text.lower():
            return "double"
        return "double" if self.prec == "double" else "real"

    def expr_type(self, u, e):
        k = e[0]
        if k == "num":
            if e[2] == "real":
                return self.lit_type(e[1])
            return "int" if e[2] == "int" else "logical"
        if k == "var":
            v = self.lookup(u, e[1])
            return "int" if v.ftype in ("int1", "logical") else v.ftype
        if k == "paren":
            return self.expr_type(u, e[1])
        if k == "un":
            return "logical" if e[1] in ("!", "!!") else self.expr_type(u, e[2])
        if k == "bin":
            op = e[1]
            if op in ("<", "<=", ">", ">=", "==", "!=", "&&", "||"):
                return "logical"
            ta, tb = self.expr_type(u, e[2]), self.expr_type(u, e[3])
            if op == "**":
                return ta if tb == "int" else self.join(ta, tb)
            return self.join(ta, tb)
        if k == "ref":
            name = e[1]
            if name in u.vars and u.vars[name].dims is not None:
                v = u.vars[name]
                return "int" if v.ftype in ("int1", "logical") else v.ftype
            if name in ("sqrt", "sin", "cos", "exp", "log", "dsqrt"):
                return self.expr_type(u, e[2][0])
            if name in ("abs", "dabs", "sign", "mod"):
                return self.expr_type(u, e[2][0])
            if name in ("max", "min", "dmax1", "dmin1", "amax1", "amin1"):
                t = self.expr_type(u, e[2][0])
                for a in e[2][1:]:
                    t = self.join(t, self.expr_type(u, a))
                return t
            if name == "dble":
                return "double"
            if name in ("real", "float"):
                return "real" if self.prec == "single" else "double"
            if name == "int":
                return "int"
            raise TranslateError(f"{u.name}: unknown function {name}")
        raise TranslateError(f"bad node {e}")

    @staticmethod
    def join(a, b):
        order = {"logical": 0, "int": 1, "real": 2, "double": 3}
        return a if order[a] >= order[b] else b

    def lookup(self, u, name):
        if name not in u.vars:
            raise TranslateError(f"{u.name}: undeclared {name}")
        return u.vars[name]

    # ---- emit expressions ------------------------------------------------
    def lit(self, text):
        t = text.lower()
        if "d" in t:
            t = t.replace("d", "e")
            return self.fix_dot(t)
        t = self.fix_dot(t)
        if self.prec == "single":
            return t + "f"
        return t

    @staticmethod
    def fix_dot(t):
        # '1.e-11' and '1.' are valid C; '.5' too.  Make sure it is floating.
        if "." not in t and "e" not in t:
            return t + ".0"
        if "." not in t:
            # e.g. 1e-6 -> fine in C
            return t
        return t

    def scal(self, u, name):
        v = self.lookup(u, name)
        if v.is_arg:
            return f"(*{name})"
        return name

    def index_expr(self, u, v, args):
        if len(args) != len(v.dims):
            raise TranslateError(f"{u.name}: rank mismatch for {v.name}")
        terms = None
        for (lo, hi), a in reversed(list(zip(v.dims, args))):
            lo_c = self.emit(u, parse_expr(lo))
            a_c = self.emit(u, a)
            off = f"((long)({a_c}) - (long)({lo_c}))"
            if terms is None:
                terms = off
            else:
                ext = f"((long)({self.emit(u, parse_expr(hi))}) - (long)({lo_c}) + 1)"
                terms = f"({off} + {ext} * {terms})"
        return terms

    def emit(self, u, e):
        k = e[0]
        if k == "num":
            return self.lit(e[1]) if e[2] == "real" else e[1]
        if k == "var":
            return self.scal(u, e[1])
        if k == "paren":
            return "(" + self.emit(u, e[1]) + ")"
        if k == "un":
            return f"({e[1]}{self.emit(u, e[2])})"
        if k == "bin":
            op = e[1]
            if op == "**":
                base = self.emit(u, e[2])
                expn = e[3]
                if expn[0] == "num" and expn[2] == "int":
                    n = int(expn[1])
                    tb = self.expr_type(u, e[2])
                    fn = {"int": "ipow", "real": "rpowi", "double": "dpowi"}[tb]
                    if tb == "real" and self.prec == "double":
                        fn = "dpowi"
                    return f"{fn}{n}({base})" if n in (2, 3, 4) else f"{fn}({base},{n})"
                tb = self.expr_type(u, e[2])
                te = self.expr_type(u, expn)
                t = self.join(tb, te)
                if t == "real" and self.prec == "single":
                    return f"powf({base},{self.emit(u, expn)})"
                return f"pow({base},{self.emit(u, expn)})"
            a = self.emit(u, e[2])
            b = self.emit(u, e[3])
            return f"({a} {op} {b})"
        if k == "ref":
            name, args = e[1], e[2]
            if name in u.vars and u.vars[name].dims is not None:
                v = u.vars[name]
                idx = self.index_expr(u, v, args)
                return f"{name}[{idx}]"
            return self.emit_intrinsic(u, name, args)
        raise TranslateError(f"bad node {e}")

    def emit_intrinsic(self, u, name, args):
        t = self.expr_type(u, ("ref", name, args))
        cargs = [self.emit(u, a) for a in args]
        if name in ("abs", "dabs"):
            if t == "int":
                return f"abs({cargs[0]})"
            return f"fabsf({cargs[0]})" if t == "real" and self.prec == "single" else f"fabs({cargs[0]})"
        if name in ("sqrt", "dsqrt", "sin", "cos", "exp", "log"):
            base = name[1:] if name == "dsqrt" else name
            if t == "real" and self.prec == "single":
                return f"{base}f({cargs[0]})"
            return f"{base}({cargs[0]})"
        if name in ("max", "min", "dmax1", "dmin1", "amax1", "amin1"):
            fn = "FMAX" if "max" in name else "FMIN"
            ct = self.ctype("double" if t == "double" else t)
            # fold left: max(a,b,c) = max(max(a,b),c)
            acc = f"(({ct})({cargs[0]}))"
            for c in cargs[1:]:
                acc = f"{fn}({acc}, (({ct})({c})))"
            return acc
        if name == "sign":
            if t == "int":
                return f"isign({cargs[0]},{cargs[1]})"
            return f"copysign({cargs[0]},{cargs[1]})" if self.prec == "double" or t == "double" else f"copysignf({cargs[0]},{cargs[1]})"
        if name == "mod":
            return f"({cargs[0]} % {cargs[1]})"
        if name == "dble":
            return f"((double)({cargs[0]}))"
        if name in ("real", "float"):
            return f"(({self.real_c})({cargs[0]}))"
        if name == "int":
            return f"((int)({cargs[0]}))"
        raise TranslateError(f"intrinsic {name}")

    # ---- statements ------------------------------------------------------
    def parse_units(self, stmts, fname):
        units, cur = [], None
        for line, s in stmts:
            low = s.lower()
            m = re.match(r"subroutine\s+([a-z_0-9]+)\s*\((.*)\)\s*$", low)
            if m:
                args = [a.strip() for a in m.group(2).split(",") if a.strip()]
                cur = Unit(m.group(1), args, fname, line)
                units.append(cur)
                continue
            if cur is None:
                raise TranslateError(f"{fname}:{line}: statement outside subroutine")
            if re.fullmatch(r"end(\s+subroutine.*)?", low):
                cur = None
                continue
            if low == "implicit none":
                continue
            m = re.match(r"(integer\*1|integer|real\*8|real|logical|double\s+precision)\s+(.*)$", low)
            if m and not re.match(r"(integer|real|logical)\s*=", low):
                ftype = {"integer*1": "int1", "integer": "int", "real": "real",
                         "real*8": "double", "logical": "logical"}.get(m.group(1), "double")
                for item in split_top(m.group(2), ","):
                    item = item.strip()
                    mm = re.match(r"([a-z_][a-z_0-9]*)\s*(\((.*)\))?$", item)
                    if not mm:
                        raise TranslateError(f"{fname}:{line}: decl {item!r}")
                    v = Var(mm.group(1), ftype)
                    if mm.group(2):
                        dims = []
                        for d in split_top(mm.group(3), ","):
                            if ":" in d:
                                lo, hi = d.split(":")
                            else:
                                lo, hi = "1", d
                            dims.append((lo.strip(), hi.strip()))
                        v.dims = dims
                    cur.vars[v.name] = v
                continue
            m = re.match(r"parameter\s*\((.*)\)\s*$", low)
            if m:
                for item in split_top(m.group(1), ","):
                    nm, ex = item.split("=", 1)
                    cur.params.append((nm.strip(), ex.strip()))
                continue
            cur.body.append((line, s))
        for u in units:
            for a in u.args:
                if a not in u.vars:
                    raise TranslateError(f"{u.name}: undeclared argument {a}")
                u.vars[a].is_arg = True
            for nm, _ in u.params:
                u.vars[nm].is_param = True
        return units

    def cname(self, name):
        return name.lower() + "_"

    def signature(self, u):
        parts = []
        for a in u.args:
            v = u.vars[a]
            parts.append(f"{self.ctype(v.ftype)} *{a}")
        return f"void {self.cname(u.name)}({', '.join(parts)})"

    def translate_unit(self, u, protos):
        out = [f"/* {u.src}:{u.line} */", self.signature(u), "{"]
        # locals
        for name, v in u.vars.items():
            if v.is_arg or v.dims is not None:
                continue
            out.append(f"  {self.ctype(v.ftype)} {name};")
        for nm, ex in u.params:
            out.append(f"  {nm} = {self.conv(u, u.vars[nm], parse_expr(ex))};")
        for name, v in u.vars.items():
            if v.is_arg or v.dims is None:
                continue
            size = " * ".join(
                f"((long)({self.emit(u, parse_expr(hi))}) - (long)({self.emit(u, parse_expr(lo))}) + 1)"
                for lo, hi in v.dims)
            out.append(f"  {self.ctype(v.ftype)} {name}[{size}];")
        out.append("  long _lo_, _hi_;")
        out.append("  (void)_lo_; (void)_hi_;")
        depth = 1
        stack = []
        loopid = [0]

        def ind():
            return "  " * depth

        for line, s in u.body:
            low = s.lower().strip()
            try:
                m = re.match(r"do\s+([a-z_][a-z_0-9]*)\s*=\s*(.*)$", low)
                if m and not re.match(r"do\s+\d", low):
                    var = m.group(1)
                    bounds = split_top(m.group(2), ",")
                    lo_c = self.emit(u, parse_expr(bounds[0]))
                    hi_c = self.emit(u, parse_expr(bounds[1]))
                    lid = loopid[0]
                    loopid[0] += 1
                    if len(bounds) == 3:
                        st_c = self.emit(u, parse_expr(bounds[2]))
                        out.append(f"{ind()}{{ long _s{lid} = {st_c}; long _t{lid} = ((long)({hi_c}) - (long)({lo_c}) + _s{lid}) / _s{lid};")
                        out.append(f"{ind()}  for ({self.scal(u, var)} = {lo_c}; _t{lid} > 0; _t{lid}--, {self.scal(u, var)} += _s{lid}) {{")
                    else:
                        out.append(f"{ind()}{{ long _h{lid} = {hi_c};")
                        out.append(f"{ind()}  for ({self.scal(u, var)} = {lo_c}; {self.scal(u, var)} <= _h{lid}; {self.scal(u, var)}++) {{")
                    stack.append("do")
                    depth += 1
                    continue
                if low in ("enddo", "end do"):
                    if not stack or stack.pop() != "do":
                        raise TranslateError("unbalanced enddo")
                    depth -= 1
                    out.append(f"{ind()}  }} }}")
                    continue
                m = re.match(r"if\s*\((.*)\)\s*then$", low)
                if m and balanced_if(low):
                    out.append(f"{ind()}if ({self.cond(u, m.group(1))}) {{")
                    stack.append("if")
                    depth += 1
                    continue
                m = re.match(r"else\s*if\s*\((.*)\)\s*then$", low)
                if m:
                    out.append(f"{'  ' * (depth - 1)}}} else if ({self.cond(u, m.group(1))}) {{")
                    continue
                if low == "else":
                    out.append(f"{'  ' * (depth - 1)}}} else {{")
                    continue
                if low in ("endif", "end if"):
                    if not stack or stack.pop() != "if":
                        raise TranslateError("unbalanced endif")
                    depth -= 1
                    out.append(f"{ind()}}}")
                    continue
                if low.startswith("if") and re.match(r"if\s*\(", low):
                    cond, rest = split_logical_if(s)
                    out.append(f"{ind()}if ({self.cond(u, cond)}) {{")
                    depth += 1
                    out.append(self.simple_stmt(u, rest, ind()))
                    depth -= 1
                    out.append(f"{ind()}}}")
                    continue
                out.append(self.simple_stmt(u, s, ind()))
            except TranslateError as exc:
                raise TranslateError(f"{u.src}:{line}: {exc}  [{s}]")
        if stack:
            raise TranslateError(f"{u.name}: unclosed block")
        out.append("}")
        protos.append(self.signature(u) + ";")
        return "\n".join(out)

    def cond(self, u, text):
        return self.emit(u, parse_expr(text))

    def conv(self, u, var, e):
        """Emit e converted to var's type (Fortran assignment semantics)."""
        c = self.emit(u, e)
        te = self.expr_type(u, e)
        if var.ftype in ("int", "int1", "logical") and te in ("real", "double"):
            return f"({self.ctype(var.ftype)})({c})"  # truncation toward zero
        return c

    def simple_stmt(self, u, s, ind):
        low = s.lower().strip()
        if low == "return":
            return f"{ind}return;"
        if low == "exit":
            return f"{ind}break;"
        if low == "continue":
            return f"{ind};"
        m = re.match(r"call\s+([a-z_0-9]+)\s*\((.*)\)\s*$", low)
        if m:
            args = [a.strip() for a in split_top(m.group(2), ",")]
            cargs = [self.actual_arg(u, a) for a in args]
            u.calls.append((m.group(1), [parse_expr(a) for a in args]))
            return f"{ind}{self.cname(m.group(1))}({', '.join(cargs)});"
        # assignment
        lhs, rhs = split_assign(s)
        le = parse_expr(lhs)
        re_ = parse_expr(rhs)
        if le[0] == "var":
            v = self.lookup(u, le[1])
            u.written.add(le[1])
            return f"{ind}{self.scal(u, le[1])} = {self.conv(u, v, re_)};"
        if le[0] == "ref":
            v = self.lookup(u, le[1])
            u.written.add(le[1])
            return f"{ind}{self.emit(u, le)} = {self.conv(u, v, re_)};"
        raise TranslateError(f"bad assignment {s}")

    def actual_arg(self, u, text):
        e = parse_expr(text)
        if e[0] == "var":
            v = self.lookup(u, e[1])
            if v.dims is not None or v.is_arg:
                return e[1]
            if v.is_param:
                return f"&({self.ctype(v.ftype)}){{{e[1]}}}"
            return f"&{e[1]}"
        if e[0] == "ref" and e[1] in u.vars and u.vars[e[1]].dims is not None:
            return f"&{self.emit(u, e)}"
        t = self.expr_type(u, e)
        ct = {"int": "int", "logical": "int", "real": self.real_c, "double": "double"}[t]
        return f"&({ct}){{{self.emit(u, e)}}}"


def balanced_if(low):
    """True when 'if (...) then' has its condition closing right before 'then'."""
    m = re.match(r"if\s*\(", low)
    depth = 0
    for i in range(m.end() - 1, len(low)):
        if low[i] == "(":
            depth += 1
        elif low[i] == ")":
            depth -= 1
            if depth == 0:
                return low[i + 1:].strip() == "then"
    return False


def split_logical_if(s):
    m = re.match(r"\s*if\s*\(", s, re.IGNORECASE)
    depth = 0
    for i in range(m.end() - 1, len(s)):
        if s[i] == "(":
            depth += 1
        elif s[i] == ")":
            depth -= 1
            if depth == 0:
                return s[m.end():i], s[i + 1:].strip()
    raise TranslateError(f"bad logical if {s}")


def split_assign(s):
    depth = 0
    for i, ch in enumerate(s):
        if ch == "(":
            depth += 1
        elif ch == ")":
            depth -= 1
        elif ch == "=" and depth == 0:
            prev = s[i - 1] if i else ""
            nxt = s[i + 1] if i + 1 < len(s) else ""
            if prev not in "<>=/" and nxt != "=":
                return s[:i], s[i + 1:]
    raise TranslateError(f"no assignment in {s!r}")


PRELUDE = r"""/* Generated from the reference Fortran by oracle/f77ref.py.  Test use only. */
#include <math.h>
#include <stdlib.h>
#define FMAX(a, b) ((a) > (b) ? (a) : (b))
#define FMIN(a, b) ((a) < (b) ? (a) : (b))
static inline int isign(int a, int b) { return b >= 0 ? abs(a) : -abs(a); }
static inline double dpowi2(double x) { return x * x; }
static inline double dpowi3(double x) { return x * x * x; }
static inline double dpowi4(double x) { double y = x * x; return y * y; }
static inline float rpowi2(float x) { return x * x; }
static inline float rpowi3(float x) { return x * x * x; }
static inline float rpowi4(float x) { float y = x * x; return y * y; }
static inline int ipow2(int x) { return x * x; }
static inline int ipow3(int x) { return x * x * x; }
static inline double dpowi(double x, int n) { double r = 1.0; int m = n < 0 ? -n : n; while (m--) r *= x; return n < 0 ? 1.0 / r : r; }
static inline float rpowi(float x, int n) { float r = 1.0f; int m = n < 0 ? -n : n; while (m--) r *= x; return n < 0 ? 1.0f / r : r; }
"""


def main(argv=None):
    ap = argparse.ArgumentParser()
    ap.add_argument("--precision", choices=["double", "single"], default="double")
    ap.add_argument("--sig-json", help="also write argument signatures as JSON")
    ap.add_argument("out")
    ap.add_argument("sources", nargs="+")
    a = ap.parse_args(argv)
    tr = Translator(a.precision)
    protos, bodies, sigs = [], [], {}
    all_units = {}
    for src in a.sources:
        text = open(src).read()
        for k, v in TEMPLATES[a.precision].items():
            text = text.replace(k, v)
        stmts = logical_lines(text, src)
        units = tr.parse_units(stmts, src)
        for u in units:
            bodies.append(tr.translate_unit(u, protos))
            all_units[u.name] = u
    # propagate "written" through calls until nothing changes
    changed = True
    while changed:
        changed = False
        for u in all_units.values():
            for callee, actuals in u.calls:
                cu = all_units.get(callee)
                if cu is None:
                    continue
                for formal, act in zip(cu.args, actuals):
                    if formal in cu.written and act[0] in ("var", "ref") and act[1] not in u.written:
                        u.written.add(act[1])
                        changed = True
    for u in all_units.values():
        sigs[tr.cname(u.name)] = {
            "src": f"{u.src}:{u.line}",
            "args": [[a_, u.vars[a_].ftype, bool(u.vars[a_].dims), a_ in u.written]
                     for a_ in u.args],
        }
    with open(a.out, "w") as f:
        f.write(PRELUDE)
        f.write("\n".join(protos) + "\n\n")
        f.write("\n\n".join(bodies) + "\n")
    if a.sig_json:
        import json
        with open(a.sig_json, "w") as f:
            json.dump(sigs, f, indent=1)
    return 0


if __name__ == "__main__":
    sys.exit(main())
