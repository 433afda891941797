"""Runs fixed-form Fortran 77 subroutines in Python with the arithmetic a
Fortran compiler gives them on an IEEE machine, to produce reference outputs
from the reference's own source where no Fortran compiler exists.

Test infrastructure only: the fixture generators beside this file use it to
run the reference's subroutines on small inputs and commit the outputs as
fixtures; nothing in the library or the benchmark imports it.

The translator turns each subroutine into a Python function:

* REAL*8 values are Python floats (IEEE binary64); a REAL*4 result is the
  binary64 result rounded to binary32 (for +, -, *, / and sqrt the binary64
  result rounded once equals the correctly rounded binary32 result, since
  53 >= 2*24 + 2); REAL*4 literals are the decimal rounded to nearest
  binary32; mixed REAL*4 / REAL*8 operations widen the REAL*4 operand;
* expressions are evaluated in source order with Fortran precedence (** right
  associative above unary minus, * and / left associative, then + and -);
  constant subexpressions are folded with the same rules, as the compiler
  folds them; no multiply-add is fused;
* x**n with an integer n is the binary powering of libgcc's __powidf2
  (n = 2: x*x; n = 3: x*(x*x)); integer division truncates toward zero;
* COMMON blocks are shared storage (one list per member, laid out as the
  first unit that declares the block lays it out, checked against every
  other unit); arguments pass by reference (an array element passes the
  array from that element on, sequence association); local arrays are
  static; local scalars start at zero;
* DO loops take their trip count once ((m2 - m1 + m3) / m3, at least 0) and
  leave the variable at m1 + trip*m3; a GOTO is supported where it jumps to
  the statement right after its enclosing DO loop (a loop exit).

Supported statements: IMPLICIT, PARAMETER, type declarations (REAL*8,
REAL*4, REAL, DOUBLE PRECISION, INTEGER, LOGICAL, CHARACTER), DIMENSION,
COMMON, assignment, DO / ENDDO / labelled DO (shared terminal labels
included), CONTINUE, block and logical IF, CALL, RETURN, STOP, GOTO (loop
exits), and PRINT / WRITE / FORMAT as no-ops.  Anything else raises
NotImplementedError naming the statement.
"""
import math
import re
from fractions import Fraction

import numpy as np

# ----------------------------------------------------------------- numerics


def r4(x):
    """binary64 -> binary32, round to nearest even."""
    return float(np.float32(x))


def dec_to_r4(text):
    """A decimal literal rounded to the nearest binary32 (ties to even)."""
    fr = Fraction(text)
    x = np.float32(float(fr))
    best = None
    for c in (np.nextafter(x, np.float32(-np.inf)), x, np.nextafter(x, np.float32(np.inf))):
        d = abs(Fraction(float(c)) - fr)
        even = (int(np.array(c, dtype=np.float32).view(np.uint32)) & 1) == 0
        key = (d, not even)
        if best is None or key < best[0]:
            best = (key, float(c))
    return best[1]


def idiv(a, b):
    q = abs(a) // abs(b)
    return q if (a >= 0) == (b > 0) else -q


def ipow(a, n):
    """Integer a**n; a negative n gives 1/(a**-n) truncated toward zero."""
    if n >= 0:
        return a ** n
    if a == 0:
        raise ZeroDivisionError("0**negative")
    if a == 1:
        return 1
    if a == -1:
        return 1 if n % 2 == 0 else -1
    return 0


def powi(x, n, rnd=None):
    """libgcc __powidf2 / __powisf2: binary powering with one rounding per
    multiplication; rnd rounds each product (REAL*4)."""
    m = -n if n < 0 else n
    r = x if m % 2 else 1.0
    while True:
        m >>= 1
        if not m:
            break
        x = x * x if rnd is None else rnd(x * x)
        if m % 2:
            r = r * x if rnd is None else rnd(r * x)
    if n < 0:
        r = 1.0 / r if rnd is None else rnd(1.0 / r)
    return r


def trip(a, b, s):
    if s == 0:
        raise ZeroDivisionError("DO step 0")
    return max(0, idiv(b - a + s, s))


def nint(x):
    return int(math.floor(x + 0.5)) if x >= 0 else -int(math.floor(-x + 0.5))


class FortranStop(Exception):
    pass


# ----------------------------------------------------------------- source

def read_units(path):
    """[(kind, name, args, [(label, text, lineno)])]: the program units of a
    fixed-form file with comments removed, continuation lines joined, text
    past column 72 dropped, blanks outside strings removed and letters
    outside strings lower-cased."""
    stmts = []
    for lineno, raw in enumerate(open(path, errors="replace"), 1):
        line = raw.rstrip("\n").rstrip("\r")
        if not line.strip():
            continue
        if line[0] in "cC*!dD" or line.lstrip().startswith("!"):
            continue
        line = line[:72]
        if line[0] == "&":   # continuation marked in column 1 (a g77 extension)
            label, cont, body = "", "&", line[1:]
        else:
            label, cont, body = line[:5].strip(), (line[5] if len(line) > 5 else " "), line[6:]
        body = _strip_comment(body)
        if cont not in (" ", "0"):
            if not stmts:
                raise ValueError("continuation without a statement at line %d" % lineno)
            stmts[-1][1] += body
            continue
        stmts.append([int(label) if label else None, body, lineno])
    out = []
    for s in stmts:
        s[1] = _squeeze(s[1])
        if s[1]:
            out.append(tuple(s))
    units, cur = [], []
    for s in out:
        cur.append(s)
        if s[1] == "end":
            units.append(cur)
            cur = []
    if cur:
        raise ValueError("unit without END")
    res = []
    for u in units:
        m = re.match(r"^subroutine([a-z]\w*)(?:\((.*)\))?$", u[0][1])
        f = re.match(r"^(real\*8|doubleprecision|real\*4|real|integer|logical)?function([a-z]\w*)\((.*)\)$",
                     u[0][1])
        if m:
            args = [a for a in (m.group(2) or "").split(",") if a]
            res.append(("subroutine", m.group(1), args, u[1:-1]))
        elif f:
            args = [a for a in f.group(3).split(",") if a]
            t = {"real*8": "d", "doubleprecision": "d", "real*4": "r", "real": "r", "integer": "i",
                 "logical": "l"}.get(f.group(1))
            res.append(("function:%s" % (t or ""), f.group(2), args, u[1:-1]))
        elif re.match(r"^program[a-z]\w*$", u[0][1]):
            res.append(("program", None, [], u[1:-1]))
        else:
            res.append(("program", None, [], u[:-1]))
    return res


def _strip_comment(s):
    q = False
    for i, ch in enumerate(s):
        if ch == "'":
            q = not q
        elif ch == "!" and not q:
            return s[:i]
    return s


def _squeeze(s):
    out, q = [], False
    for ch in s:
        if ch == "'":
            q = not q
            out.append(ch)
        elif q:
            out.append(ch)
        elif ch not in " \t":
            out.append(ch.lower())
    return "".join(out)


def split_top(s, sep=","):
    parts, depth, q, start = [], 0, False, 0
    for i, ch in enumerate(s):
        if ch == "'":
            q = not q
        elif q:
            continue
        elif ch == "(":
            depth += 1
        elif ch == ")":
            depth -= 1
        elif ch == sep and depth == 0:
            parts.append(s[start:i])
            start = i + 1
    parts.append(s[start:])
    return parts


def find_top(s, ch):
    depth, q = 0, False
    for i, c in enumerate(s):
        if c == "'":
            q = not q
        elif q:
            continue
        elif c == "(":
            depth += 1
        elif c == ")":
            depth -= 1
        elif c == ch and depth == 0:
            return i
    return -1


def match_paren(s, i):
    depth = 0
    for j in range(i, len(s)):
        if s[j] == "(":
            depth += 1
        elif s[j] == ")":
            depth -= 1
            if depth == 0:
                return j
    raise ValueError("unbalanced parentheses: " + s)


# ----------------------------------------------------------------- expressions

_DOTOPS = ("eq", "ne", "lt", "le", "gt", "ge", "and", "or", "not", "eqv", "neqv", "true", "false")
_NUM = re.compile(r"(\d+\.\d*|\.\d+|\d+)([ed][+-]?\d+)?")


def tokenize(s):
    toks, i, n = [], 0, len(s)
    while i < n:
        c = s[i]
        if c == "." and i + 1 < n and s[i + 1].isalpha():
            m = re.match(r"\.([a-z]+)\.", s[i:])
            if m and m.group(1) in _DOTOPS:
                toks.append(("op", m.group(1)))
                i += m.end()
                continue
        if c.isdigit() or (c == "." and i + 1 < n and s[i + 1].isdigit()):
            j = i
            while j < n and s[j].isdigit():
                j += 1
            is_real = False
            if j < n and s[j] == "." and not re.match(r"\.(%s)\." % "|".join(_DOTOPS), s[j:]):
                j += 1
                while j < n and s[j].isdigit():
                    j += 1
                is_real = True
            m = re.match(r"[ed][+-]?\d+", s[j:])
            if m:
                exp = m.group(0)
                j += len(exp)
                is_real = True
            text = s[i:j]
            if not is_real:
                toks.append(("int", int(text)))
            elif "d" in text:
                toks.append(("r8", float(text.replace("d", "e"))))
            else:
                toks.append(("r4", dec_to_r4(text)))
            i = j
            continue
        if c.isalpha():
            m = re.match(r"[a-z]\w*", s[i:])
            toks.append(("name", m.group(0)))
            i += m.end()
            continue
        if c == "'":
            j = s.index("'", i + 1)
            toks.append(("str", s[i + 1:j]))
            i = j + 1
            continue
        if s.startswith("**", i):
            toks.append(("op", "**"))
            i += 2
            continue
        if c in "+-*/(),:":
            toks.append(("op", c))
            i += 1
            continue
        raise NotImplementedError("cannot tokenize %r in %r" % (s[i:], s))
    return toks


class Parser:
    """Fortran expression -> tree: ('num', type, value) | ('str', s) |
    ('name', n) | ('ref', n, [args]) | ('un', op, x) | ('bin', op, a, b)."""

    def __init__(self, text):
        self.t = tokenize(text)
        self.i = 0

    def peek(self, k=0):
        return self.t[self.i + k] if self.i + k < len(self.t) else (None, None)

    def take(self, kind=None, val=None):
        tok = self.peek()
        if kind and tok[0] != kind or val is not None and tok[1] != val:
            raise ValueError("expected %s %s, got %s" % (kind, val, tok))
        self.i += 1
        return tok

    def parse(self):
        e = self.p_eqv()
        if self.i != len(self.t):
            raise ValueError("trailing tokens %s" % (self.t[self.i:],))
        return e

    def p_eqv(self):
        a = self.p_or()
        while self.peek() in (("op", "eqv"), ("op", "neqv")):
            op = self.take()[1]
            a = ("bin", op, a, self.p_or())
        return a

    def p_or(self):
        a = self.p_and()
        while self.peek() == ("op", "or"):
            self.take()
            a = ("bin", "or", a, self.p_and())
        return a

    def p_and(self):
        a = self.p_not()
        while self.peek() == ("op", "and"):
            self.take()
            a = ("bin", "and", a, self.p_not())
        return a

    def p_not(self):
        if self.peek() == ("op", "not"):
            self.take()
            return ("un", "not", self.p_not())
        return self.p_rel()

    def p_rel(self):
        a = self.p_add()
        if self.peek()[0] == "op" and self.peek()[1] in ("eq", "ne", "lt", "le", "gt", "ge"):
            op = self.take()[1]
            a = ("bin", op, a, self.p_add())
        return a

    def p_add(self):
        if self.peek() in (("op", "+"), ("op", "-")):
            op = self.take()[1]
            a = self.p_mul()
            if op == "-":
                a = ("un", "-", a)
        else:
            a = self.p_mul()
        while self.peek() in (("op", "+"), ("op", "-")):
            op = self.take()[1]
            a = ("bin", op, a, self.p_mul())
        return a

    def p_mul(self):
        a = self.p_pow()
        while self.peek() in (("op", "*"), ("op", "/")):
            op = self.take()[1]
            a = ("bin", op, a, self.p_pow())
        return a

    def p_pow(self):
        a = self.p_prim()
        if self.peek() == ("op", "**"):
            self.take()
            if self.peek() in (("op", "+"), ("op", "-")):   # x**-2 (an extension)
                op = self.take()[1]
                b = self.p_pow()
                b = ("un", "-", b) if op == "-" else b
            else:
                b = self.p_pow()
            a = ("bin", "**", a, b)
        return a

    def p_prim(self):
        kind, v = self.peek()
        if kind in ("int", "r4", "r8"):
            self.take()
            return ("num", {"int": "i", "r4": "r", "r8": "d"}[kind], v)
        if kind == "str":
            self.take()
            return ("str", v)
        if (kind, v) == ("op", "true") or (kind, v) == ("op", "false"):
            self.take()
            return ("num", "l", v == "true")
        if kind == "name":
            self.take()
            if self.peek() == ("op", "("):
                self.take()
                args = []
                if self.peek() != ("op", ")"):
                    args.append(self.p_eqv())
                    while self.peek() == ("op", ","):
                        self.take()
                        args.append(self.p_eqv())
                self.take("op", ")")
                return ("ref", v, args)
            return ("name", v)
        if (kind, v) == ("op", "("):
            self.take()
            e = self.p_eqv()
            self.take("op", ")")
            return e
        raise ValueError("unexpected token %s" % ((kind, v),))


def parse_expr(text):
    return Parser(text).parse()


# ----------------------------------------------------------------- statements

def classify(label, s, lineno):
    """One executable statement -> a tuple whose first item is its kind."""
    if s == "continue":
        return ("continue",)
    if s == "return":
        return ("return",)
    if s == "stop" or s.startswith("stop") and find_top(s, "=") < 0:
        return ("stop",)
    if s in ("enddo",):
        return ("enddo",)
    if s in ("endif",):
        return ("endif",)
    if s == "else":
        return ("else",)
    if s.startswith("elseif(") and s.endswith("then"):
        j = match_paren(s, 6)
        return ("elseif", parse_expr(s[7:j]))
    if s.startswith("if(") :
        j = match_paren(s, 2)
        rest = s[j + 1:]
        cond = parse_expr(s[3:j])
        if rest == "then":
            return ("ifthen", cond)
        if rest:
            return ("logif", cond, classify(None, rest, lineno))
    m = re.match(r"^do(\d+)?,?([a-z]\w*)=(.*)$", s)
    if m and len(split_top(m.group(3))) in (2, 3):
        parts = [parse_expr(p) for p in split_top(m.group(3))]
        step = parts[2] if len(parts) == 3 else ("num", "i", 1)
        return ("do", int(m.group(1)) if m.group(1) else None, m.group(2), parts[0], parts[1], step)
    if s.startswith("goto") or s.startswith("go to"):
        return ("goto", int(s[4:]))
    if s.startswith("call") and find_top(s, "=") < 0:
        m = re.match(r"^call([a-z]\w*)(?:\((.*)\))?$", s)
        args = [parse_expr(a) for a in split_top(m.group(2))] if m.group(2) else []
        return ("call", m.group(1), args)
    if s.startswith(("print", "write(", "format(", "open(", "close(", "rewind", "backspace", "inquire")) \
            and find_top(s, "=") < 0:
        return ("io",)
    if s.startswith("read*"):
        items = s[5:].lstrip(",")
        return ("read", [parse_expr(x) for x in split_top(items)] if items else [])
    if s.startswith("read(") and find_top(s, "=") < 0:
        return ("readunit", lineno)
    k = find_top(s, "=")
    if k > 0:
        return ("assign", parse_expr(s[:k]), parse_expr(s[k + 1:]))
    raise NotImplementedError("line %d: statement %r" % (lineno, s))


def goto_targets(node):
    """Labels that GOTO statements anywhere inside node jump to."""
    k = node[0]
    if k == "goto":
        return {node[1]}
    if k == "logif":
        return goto_targets(node[2])
    if k == "do":
        out = set()
        for _, n in node[5]:
            out |= goto_targets(n)
        return out
    if k == "if":
        out = set()
        for _, body in node[1]:
            for _, n in body:
                out |= goto_targets(n)
        return out
    return set()


def labels_in(items):
    out = set()
    for lab, n in items:
        if lab is not None:
            out.add(lab)
        if n[0] == "do":
            out |= labels_in(n[5])
        elif n[0] == "if":
            for _, body in n[1]:
                out |= labels_in(body)
    return out


def build_blocks(stmts):
    """Flat executable statements -> nested blocks.  Each item is
    (label, node); 'do' nodes get a body list, 'if' nodes a list of
    (cond, body) branches and an else body."""
    root = []
    stack = [("root", root, None)]

    def close_dos(label):
        while label is not None and stack[-1][0] == "do" and stack[-1][2] == label:
            _, body, _, node = stack.pop()
            stack[-1][1].append(node)

    for label, node, lineno in stmts:
        kind = node[0]
        if kind == "do":
            body = []
            dnode = (label, ("do", node[2], node[3], node[4], node[5], body, lineno))
            stack.append(("do", body, node[1], dnode))
            if node[1] is None:
                stack[-1] = ("do", body, "enddo", dnode)
            continue
        if kind == "enddo":
            if stack[-1][0] != "do" or stack[-1][2] != "enddo":
                raise ValueError("line %d: ENDDO without DO" % lineno)
            _, body, _, dnode = stack.pop()
            stack[-1][1].append(dnode)
            close_dos(label)
            continue
        if kind == "ifthen":
            branches = [[node[1], []]]
            inode = (label, ("if", branches, None, lineno))
            stack.append(("if", branches[0][1], None, inode, branches))
            continue
        if kind in ("elseif", "else"):
            top = stack.pop()
            if top[0] != "if":
                raise ValueError("line %d: ELSE outside IF" % lineno)
            branches = top[4]
            if kind == "elseif":
                branches.append([node[1], []])
                stack.append(("if", branches[-1][1], None, top[3], branches))
            else:
                branches.append([None, []])
                stack.append(("if", branches[-1][1], None, top[3], branches))
            continue
        if kind == "endif":
            top = stack.pop()
            if top[0] != "if":
                raise ValueError("line %d: ENDIF outside IF" % lineno)
            stack[-1][1].append(top[3])
            close_dos(label)
            continue
        stack[-1][1].append((label, node))
        close_dos(label)
    if len(stack) != 1:
        raise ValueError("unclosed block: %s" % (stack[-1][0],))
    return root


# ----------------------------------------------------------------- units

_INTRINSIC_TYPES = {
    "dble": "d", "dfloat": "d", "float": "r", "real": "r", "sngl": "r", "int": "i", "ifix": "i",
    "idint": "i", "nint": "i", "idnint": "i",
}
_MATH = {"sqrt": "sqrt", "dsqrt": "sqrt", "exp": "exp", "dexp": "exp", "log": "log", "dlog": "log",
         "alog": "log", "log10": "log10", "dlog10": "log10", "alog10": "log10", "sin": "sin", "dsin": "sin",
         "cos": "cos", "dcos": "cos", "tan": "tan", "dtan": "tan", "atan": "atan", "datan": "atan",
         "acos": "acos", "dacos": "acos", "asin": "asin", "dasin": "asin", "sinh": "sinh", "dsinh": "sinh",
         "cosh": "cosh", "dcosh": "cosh", "tanh": "tanh", "dtanh": "tanh"}
_MINMAX = {"max": None, "min": None, "max0": "i", "min0": "i", "amax1": "r", "amin1": "r",
           "dmax1": "d", "dmin1": "d"}


class Var:
    def __init__(self, name, typ):
        self.name, self.typ = name, typ
        self.dims = None          # [(lo_tree, hi_tree or None)]
        self.kind = "local"       # local | common | dummy
        self.common = None        # (block, index)
        self.used_as_actual = False


class Unit:
    def __init__(self, name, args, stmts, commons, result=None):
        self.name, self.args = name, args
        self.result = result      # a FUNCTION's result variable
        self.implicit = {c: ("i" if "i" <= c <= "n" else "r") for c in "abcdefghijklmnopqrstuvwxyz"}
        self.params = {}
        self.vars = {}
        self.commons = commons
        self.exec = []
        self._declare(stmts)

    def typ_of(self, n):
        if n in self.params:
            return self.params[n][0]
        if n in self.vars:
            return self.vars[n].typ
        return self.implicit[n[0]]

    def var(self, n):
        if n not in self.vars:
            self.vars[n] = Var(n, self.implicit[n[0]])
        return self.vars[n]

    def _declare(self, stmts):
        for a in self.args:
            self.var(a).kind = "dummy"
        execs = []
        for label, s, lineno in stmts:
            if s.startswith("implicit"):
                if s == "implicitnone":
                    continue
                m = re.match(r"^implicit(real\*8|doubleprecision|real\*4|real|integer|logical)\((.*)\)$", s)
                if not m:
                    raise NotImplementedError("line %d: %r" % (lineno, s))
                t = {"real*8": "d", "doubleprecision": "d", "real*4": "r", "real": "r", "integer": "i",
                     "logical": "l"}[m.group(1)]
                for rng in m.group(2).split(","):
                    lo, hi = (rng.split("-") + [rng])[:2]
                    for c in range(ord(lo), ord(hi) + 1):
                        self.implicit[chr(c)] = t
                for v in self.vars.values():
                    if v.kind == "dummy" and not getattr(v, "explicit", False):
                        v.typ = self.implicit[v.name[0]]
                continue
            if s.startswith("parameter("):
                for item in split_top(s[10:-1]):
                    n, e = item.split("=", 1)
                    t = self.typ_of(n)
                    val = self.const_eval(parse_expr(e))
                    self.params[n] = (t, convert_const(val, t))
                continue
            m = re.match(r"^(real\*8|doubleprecision|real\*4|real|integer\*4|integer|logical|character(?:\*\d+)?)(.*)$", s)
            if m and not s.startswith("realfunction") and find_top(s, "=") < 0:
                t = {"real*8": "d", "doubleprecision": "d", "real*4": "r", "real": "r", "integer": "i",
                     "integer*4": "i", "logical": "l"}.get(m.group(1), "c")
                for ent in split_top(m.group(2)):
                    self._entity(ent, t)
                continue
            if s.startswith("dimension"):
                for ent in split_top(s[9:]):
                    self._entity(ent, None)
                continue
            if s.startswith("common"):
                self._common(s[6:], lineno)
                continue
            if s.startswith(("save", "data", "equivalence", "external", "intrinsic", "entry")) \
                    and find_top(s, "=") < 0:
                raise NotImplementedError("line %d: %r" % (lineno, s))
            if s.startswith("format("):
                continue
            execs.append((label, classify(label, s, lineno), lineno))
        self.exec = build_blocks(execs)

    def _entity(self, ent, t):
        m = re.match(r"^([a-z]\w*)(?:\((.*)\))?$", ent)
        v = self.var(m.group(1))
        if t is not None:
            v.typ = t
            v.explicit = True
        if m.group(2):
            dims = []
            for d in split_top(m.group(2)):
                if ":" in d:
                    lo, hi = d.split(":")
                else:
                    lo, hi = "1", d
                dims.append((parse_expr(lo), None if hi == "*" else parse_expr(hi)))
            v.dims = dims

    def _common(self, s, lineno):
        # /name/a,b,c[/name2/...]
        for m in re.finditer(r"/([a-z]\w*)/([^/]*)", s):
            blk = m.group(1)
            names = [re.match(r"[a-z]\w*", e).group(0) for e in split_top(m.group(2).rstrip(",")) if e]
            for ent in split_top(m.group(2).rstrip(",")):
                if "(" in ent:
                    self._entity(ent, None)
            for k, n in enumerate(names):
                v = self.var(n)
                v.kind, v.common = "common", (blk, k)
            self.commons.setdefault(("decl", blk), []).append((self, names))

    # constant expressions (PARAMETER values, dimension bounds)
    def const_eval(self, e):
        k = e[0]
        if k == "num":
            return (e[1], e[2])
        if k == "name":
            if e[1] in self.params:
                return self.params[e[1]]
            raise KeyError(e[1])
        if k == "un":
            t, x = self.const_eval(e[2])
            if e[1] == "-":
                return (t, -x)
            return (t, not x)
        if k == "bin":
            return fold(e[1], self.const_eval(e[2]), self.const_eval(e[3]))
        if k == "ref" and e[1] in _INTRINSIC_TYPES:
            t, x = self.const_eval(e[2][0])
            if e[1] in ("nint", "idnint"):
                return ("i", nint(x))
            rt = _INTRINSIC_TYPES[e[1]]
            return (rt, convert_const((t, x), rt))
        raise KeyError(str(e))


def convert_const(tv, t):
    tt, x = tv
    if t == "i":
        return int(x) if tt != "i" else x
    if t == "d":
        return float(x)
    if t == "r":
        return r4(float(x))
    return x


def fold(op, a, b):
    ta, x = a
    tb, y = b
    if op in ("and", "or", "eqv", "neqv"):
        return ("l", {"and": x and y, "or": x or y, "eqv": x == y, "neqv": x != y}[op])
    t = "d" if "d" in (ta, tb) else "r" if "r" in (ta, tb) else "i"
    if op == "**":
        if tb == "i":
            if ta == "i":
                return ("i", ipow(x, y))
            return (ta, powi(float(x), y, r4 if ta == "r" else None))
        v = math.pow(float(x), float(y))
        return (t, r4(v) if t == "r" else v)
    if op in ("eq", "ne", "lt", "le", "gt", "ge"):
        if "c" in (ta, tb):
            x, y = str(x).rstrip(), str(y).rstrip()
        elif t != "i":
            x, y = float(x), float(y)
        return ("l", {"eq": x == y, "ne": x != y, "lt": x < y, "le": x <= y, "gt": x > y, "ge": x >= y}[op])
    if t == "i":
        v = {"+": x + y, "-": x - y, "*": x * y}.get(op) if op != "/" else idiv(x, y)
        return ("i", v)
    x, y = float(x), float(y)
    v = {"+": x + y, "-": x - y, "*": x * y, "/": x / y}[op]
    return (t, r4(v) if t == "r" else v)


# ----------------------------------------------------------------- code generation

class Gen:
    def __init__(self, unit, program):
        self.u, self.prog = unit, program
        self.lines = []
        self.tmp = 0
        self.ctx = []
        self.uses_goto = False

    def new(self, p="t"):
        self.tmp += 1
        return "_%s%d" % (p, self.tmp)

    # ---- storage names
    def is_array(self, n):
        return n in self.u.vars and self.u.vars[n].dims is not None

    def scalar_loc(self, n):
        """Python lvalue/rvalue text of a scalar variable."""
        v = self.u.vars.get(n) or self.u.var(n)
        if v.kind == "local":
            return "v_" + n
        return "b_%s[o_%s]" % (n, n)

    def bound(self, tree):
        code, t, c = self.expr(tree)
        return code, c

    def linear(self, n, subs):
        v = self.u.vars[n]
        if len(subs) != len(v.dims):
            raise ValueError("%s: rank mismatch in %s" % (self.u.name, n))
        terms = None
        for k in range(len(v.dims) - 1, -1, -1):
            lo_code, lo_c = self.bound(v.dims[k][0])
            s_code, st, s_c = self.expr(subs[k])
            if st != "i":
                raise ValueError("non-integer subscript of %s" % n)
            if lo_c is not None and s_c is not None:
                d = str(s_c - lo_c)
            elif lo_c is not None:
                d = "(%s - %d)" % (s_code, lo_c) if lo_c else s_code
            else:
                d = "(%s - (%s))" % (s_code, lo_code)
            if terms is None:
                terms = d
            else:
                hi_code, hi_c = self.bound(v.dims[k][1])
                if lo_c is not None and hi_c is not None:
                    ext = str(hi_c - lo_c + 1)
                else:
                    ext = "((%s) - (%s) + 1)" % (hi_code, lo_code)
                terms = "%s + %s * (%s)" % (d, ext, terms) if ext != "1" else "%s + (%s)" % (d, terms)
        return terms

    def elem(self, n, subs):
        return "b_%s[o_%s + %s]" % (n, n, self.linear(n, subs))

    # ---- expressions: (code, type, constant value or None)
    def expr(self, e):
        k = e[0]
        if k == "num":
            return (lit(e[1], e[2]), e[1], e[2])
        if k == "str":
            return (repr(e[1]), "c", e[1])
        if k == "name":
            n = e[1]
            if n in self.u.params:
                t, x = self.u.params[n]
                return (lit(t, x), t, x)
            if self.is_array(n):
                raise ValueError("%s: whole array %s in an expression" % (self.u.name, n))
            return (self.scalar_loc(n), self.u.typ_of(n), None)
        if k == "ref":
            n = e[1]
            if self.is_array(n):
                return (self.elem(n, e[2]), self.u.typ_of(n), None)
            if n in self.prog.units and self.prog.units[n].result:
                fu = self.prog.units[n]
                return ("F_%s(%s)" % (n, ", ".join(self.arg_ref(a) for a in e[2])), fu.typ_of(n), None)
            return self.intrinsic(n, e[2])
        if k == "un":
            c, t, x = self.expr(e[2])
            if e[1] == "-":
                if x is not None:
                    return (lit(t, -x), t, -x)
                return ("(-%s)" % c, t, None)
            if x is not None:
                return (lit("l", not x), "l", not x)
            return ("(not %s)" % c, "l", None)
        if k == "bin":
            return self.binop(e[1], self.expr(e[2]), self.expr(e[3]))
        raise ValueError(str(e))

    def binop(self, op, a, b):
        ca, ta, xa = a
        cb, tb, xb = b
        if xa is not None and xb is not None:
            t, v = fold(op, (ta, xa), (tb, xb))
            return (lit(t, v), t, v)
        if op in ("and", "or"):
            return ("(%s %s %s)" % (ca, op, cb), "l", None)
        if op in ("eqv", "neqv"):
            return ("(%s %s %s)" % (ca, "==" if op == "eqv" else "!=", cb), "l", None)
        t = "d" if "d" in (ta, tb) else "r" if "r" in (ta, tb) else "i"
        if op == "**":
            if tb == "i":
                if ta == "i":
                    return ("ipow(%s, %s)" % (ca, cb), "i", None)
                return ("powi(%s, %s%s)" % (ca, cb, ", r4" if ta == "r" else ""), ta, None)
            code = "math.pow(%s, %s)" % (self.to_real(ca, ta), self.to_real(cb, tb))
            return ("r4(%s)" % code if t == "r" else code, t, None)
        if op in ("eq", "ne", "lt", "le", "gt", "ge"):
            pyop = {"eq": "==", "ne": "!=", "lt": "<", "le": "<=", "gt": ">", "ge": ">="}[op]
            if "c" in (ta, tb):   # blank-padded comparison
                return ("(%s.rstrip() %s %s.rstrip())" % (ca, pyop, cb), "l", None)
            if t != "i":
                ca, cb = self.to_real(ca, ta), self.to_real(cb, tb)
            return ("(%s %s %s)" % (ca, pyop, cb), "l", None)
        if t == "i":
            if op == "/":
                return ("idiv(%s, %s)" % (ca, cb), "i", None)
            return ("(%s %s %s)" % (ca, op, cb), "i", None)
        code = "(%s %s %s)" % (self.to_real(ca, ta), op, self.to_real(cb, tb))
        return ("r4%s" % code if t == "r" else code, t, None)

    @staticmethod
    def to_real(c, t):
        return "float(%s)" % c if t == "i" else c

    def intrinsic(self, n, args):
        vals = [self.expr(a) for a in args]
        if n in _INTRINSIC_TYPES:
            (c, t, x), rt = vals[0], _INTRINSIC_TYPES[n]
            if x is not None:
                v = ("i", nint(x)) if n in ("nint", "idnint") else convert_const((t, x), rt)
                v = v if isinstance(v, tuple) else (rt, v)
                return (lit(*v), v[0], v[1])
            if n in ("nint", "idnint"):
                return ("nint(%s)" % c, "i", None)
            if rt == "i":
                return ("int(%s)" % c, "i", None)
            if rt == "d":
                return (self.to_real(c, t), "d", None)
            return ("r4(%s)" % self.to_real(c, t), "r", None)
        if n in _MATH:
            c, t, x = vals[0]
            code = "math.%s(%s)" % (_MATH[n], self.to_real(c, t))
            if t == "r":
                return ("r4(%s)" % code, "r", None)
            return (code, "d", None)
        if n in ("abs", "dabs", "iabs"):
            c, t, x = vals[0]
            return ("abs(%s)" % c, t, None)
        if n in _MINMAX:
            ts = [v[1] for v in vals]
            t = _MINMAX[n] or ("d" if "d" in ts else "r" if "r" in ts else "i")
            cs = [self.to_real(v[0], v[1]) if t != "i" else v[0] for v in vals]
            f = "max" if "max" in n else "min"
            return ("%s(%s)" % (f, ", ".join(cs)), t, None)
        if n in ("mod", "amod", "dmod"):
            (ca, ta, _), (cb, tb, _) = vals
            if ta == "i" and tb == "i":
                return ("(%s - idiv(%s, %s) * %s)" % (ca, ca, cb, cb), "i", None)
            t = "d" if "d" in (ta, tb) else "r"
            code = "math.fmod(%s, %s)" % (self.to_real(ca, ta), self.to_real(cb, tb))
            return ("r4(%s)" % code if t == "r" else code, t, None)
        if n in ("sign", "dsign", "isign"):
            (ca, ta, _), (cb, tb, _) = vals
            if ta == "i":
                return ("(abs(%s) if %s >= 0 else -abs(%s))" % (ca, cb, ca), "i", None)
            return ("math.copysign(abs(%s), %s)" % (ca, self.to_real(cb, tb)), ta, None)
        if n in ("atan2", "datan2"):
            (ca, ta, _), (cb, tb, _) = vals
            code = "math.atan2(%s, %s)" % (self.to_real(ca, ta), self.to_real(cb, tb))
            return ("r4(%s)" % code if ta == "r" else code, ta, None)
        raise NotImplementedError("%s: function %s" % (self.u.name, n))

    def convert(self, code, t, target):
        if target == t or target in ("l", "c"):
            return code
        if target == "i":
            return "int(%s)" % code
        if target == "d":
            return self.to_real(code, t)
        if target == "r":
            return code if t == "r" else "r4(%s)" % self.to_real(code, t)
        return code

    # ---- statements
    def emit(self, ind, text):
        self.lines.append("    " * ind + text)

    def block(self, items, ind):
        """A statement list.  A forward GOTO into this list (from a statement
        of it, at any depth) sets _gt to the target label; the statements
        between the jumping statement and the target run under
        `if not _gt`, and the target clears _gt."""
        if not items:
            self.emit(ind, "pass")
            return
        self.ctx.append(("list", {lab for lab, _ in items if lab is not None}))
        guard, opened, cur = None, False, ind
        for pos, (label, node) in enumerate(items):
            if guard is not None and label == guard:
                self.emit(ind, "if _gt == %d:" % guard)
                self.emit(ind + 1, "_gt = 0")
                guard, opened, cur = None, False, ind
            elif guard is not None and not opened:
                self.emit(ind, "if not _gt:")
                opened, cur = True, ind + 1
            nxt = items[pos + 1][0] if pos + 1 < len(items) else None
            self.stmt(node, cur, nxt)
            later = {lab for lab, _ in items[pos + 1:] if lab is not None}
            tg = goto_targets(node) & later
            if tg and guard is None:
                if len(tg) > 1:
                    raise NotImplementedError("%s: several forward GOTO targets" % self.u.name)
                guard = tg.pop()
        if guard is not None:
            raise NotImplementedError("%s: GOTO %d target not reached" % (self.u.name, guard))
        self.ctx.pop()

    def stmt(self, node, ind, next_label):
        k = node[0]
        if k == "assign":
            lhs, rhs = node[1], node[2]
            c, t, _ = self.expr(rhs)
            if lhs[0] == "name":
                n = lhs[1]
                tgt = self.scalar_loc(n)
                self.emit(ind, "%s = %s" % (tgt, self.convert(c, t, self.u.typ_of(n))))
            elif lhs[0] == "ref" and self.is_array(lhs[1]):
                self.emit(ind, "%s = %s" % (self.elem(lhs[1], lhs[2]), self.convert(c, t, self.u.typ_of(lhs[1]))))
            else:
                raise NotImplementedError("%s: assignment to %s" % (self.u.name, lhs))
        elif k == "do":
            _, var, a, b, s, body, lineno = node
            if self.u.var(var).dims is not None or self.u.typ_of(var) != "i":
                raise NotImplementedError("%s: DO variable %s" % (self.u.name, var))
            ta, tb, ts = self.new("a"), self.new("b"), self.new("s")
            tn = self.new("n")
            for tv, e in ((ta, a), (tb, b), (ts, s)):
                c, t, _ = self.expr(e)
                self.emit(ind, "%s = %s" % (tv, self.convert(c, t, "i")))
            self.emit(ind, "%s = trip(%s, %s, %s)" % (tn, ta, tb, ts))
            probe = self.prog.probes.get((self.u.name, lineno))
            loc = self.scalar_loc(var)
            it = "v_" + var if loc.startswith("v_") else self.new("i")
            self.emit(ind, "for %s in range(%s, %s + %s * %s, %s):" % (it, ta, ta, tn, ts, ts))
            if it != loc:
                self.emit(ind + 1, "%s = %s" % (loc, it))
            if probe:
                self.emit(ind + 1, "PROBE[%r].append(%s)" % (probe, it))
            self.ctx.append(("loop",))
            self.block(body, ind + 1)
            self.ctx.pop()
            self.emit(ind, "else:")
            self.emit(ind + 1, "%s = %s + %s * %s" % (loc, ta, tn, ts))
            # a jump that leaves this loop for a list beyond the enclosing
            # loop leaves that loop too
            out = goto_targets(("do", var, a, b, s, body, lineno)) - labels_in(body)
            for c in reversed(self.ctx):
                if c[0] == "loop":
                    if out:
                        self.emit(ind, "if _gt:")
                        self.emit(ind + 1, "break")
                    break
                if out <= c[1]:
                    break
        elif k == "read":
            targets = node[1]
            vals = self.new("r")
            types = []
            for tgt in targets:
                n = tgt[1]
                if tgt[0] == "name" and self.is_array(n):
                    raise NotImplementedError("%s: READ of a whole array" % self.u.name)
                types.append(self.u.typ_of(n))
            self.emit(ind, "%s = INPUT.read(%r)" % (vals, "".join(types)))
            for q, tgt in enumerate(targets):
                if tgt[0] == "name":
                    self.emit(ind, "%s = %s[%d]" % (self.scalar_loc(tgt[1]), vals, q))
                else:
                    self.emit(ind, "%s = %s[%d]" % (self.elem(tgt[1], tgt[2]), vals, q))
        elif k == "readunit":
            self.emit(ind, "raise NotImplementedError('READ from a unit, line %d')" % node[1])
        elif k == "if":
            branches = node[1]
            for bi, (cond, body) in enumerate(branches):
                if cond is None:
                    self.emit(ind, "else:")
                else:
                    c, t, _ = self.expr(cond)
                    self.emit(ind, "%s %s:" % ("if" if bi == 0 else "elif", c))
                self.block(body, ind + 1)
        elif k == "logif":
            c, t, _ = self.expr(node[1])
            self.emit(ind, "if %s:" % c)
            self.stmt(node[2], ind + 1, next_label)
        elif k == "continue" or k == "io":
            self.emit(ind, "pass")
        elif k == "return":
            self.emit(ind, "return v_%s" % self.u.result if self.u.result else "return")
        elif k == "stop":
            self.emit(ind, "raise FortranStop(%r)" % self.u.name)
        elif k == "goto":
            # forward jumps only: to a later statement of an enclosing list,
            # leaving the loops in between by break
            self.uses_goto = True
            self.emit(ind, "_gt = %d" % node[1])
            for c in reversed(self.ctx):
                if c[0] == "loop":
                    self.emit(ind, "break")
                    break
                if node[1] in c[1]:
                    break
            else:
                raise NotImplementedError("%s: GOTO %d has no enclosing target" % (self.u.name, node[1]))
        elif k == "call":
            self.call(node[1], node[2], ind)
        else:
            raise NotImplementedError("%s: %s" % (self.u.name, k))

    def arg_ref(self, a):
        """An actual argument inside an expression (a FUNCTION reference):
        by reference for arrays, array elements and COMMON or dummy scalars;
        a local scalar goes by value (a function that assigns it would not
        be seen: the reference's functions do not)."""
        if a[0] == "name" and a[1] not in self.u.params:
            v = self.u.var(a[1])
            if v.dims is not None or v.kind != "local":
                return "(b_%s, o_%s)" % (a[1], a[1])
            return "([v_%s], 0)" % a[1]
        if a[0] == "ref" and self.is_array(a[1]):
            return "(b_%s, o_%s + %s)" % (a[1], a[1], self.linear(a[1], a[2]))
        c, t, _ = self.expr(a)
        return "([%s], 0)" % c

    def call(self, name, args, ind):
        refs, back = [], []
        for a in args:
            if a[0] == "name" and a[1] not in self.u.params:
                n = a[1]
                v = self.u.var(n)
                if v.dims is not None or v.kind != "local":
                    refs.append("(b_%s, o_%s)" % (n, n))
                else:
                    cell = self.new("c")
                    self.emit(ind, "%s = [v_%s]" % (cell, n))
                    refs.append("(%s, 0)" % cell)
                    back.append("v_%s = %s[0]" % (n, cell))
            elif a[0] == "ref" and self.is_array(a[1]):
                refs.append("(b_%s, o_%s + %s)" % (a[1], a[1], self.linear(a[1], a[2])))
            else:
                c, t, _ = self.expr(a)
                refs.append("([%s], 0)" % c)
        self.emit(ind, "F_%s(%s)" % (name, ", ".join(refs)))
        for b in back:
            self.emit(ind, b)

    def function(self):
        """The unit as Python source: the body is generated first, so that
        every name it touches is known when the prologue binds storage and
        zeroes the local scalars."""
        u = self.u
        if u.result:
            u.var(u.result)
        self.block(u.exec, 1)
        if u.result:
            self.emit(1, "return v_%s" % u.result)
        body, self.lines = self.lines, []
        self.emit(0, "def F_%s(%s):" % (u.name, ", ".join("a_" + a for a in u.args)))
        for a in u.args:
            self.emit(1, "b_%s, o_%s = a_%s" % (a, a, a))
        for n, v in sorted(u.vars.items()):
            if v.kind == "common":
                blk, idx = v.common
                self.emit(1, "b_%s = COMMON[%r][%d]; o_%s = 0" % (n, blk, idx, n))
            elif v.kind == "local" and v.dims is not None:
                self.emit(1, "b_%s = STATIC[%r]; o_%s = 0" % (n, (u.name, n), n))
                self.prog.statics[(u.name, n)] = (v.typ, self.size_of(v))
            elif v.kind == "local":
                init = {"i": "0", "l": "False", "c": "''"}.get(v.typ, "0.0")
                self.emit(1, "v_%s = %s" % (n, init))
        if self.uses_goto:
            self.emit(1, "_gt = 0")
        return "\n".join(self.lines + body)

    def size_of(self, v):
        n = 1
        for lo, hi in v.dims:
            a = self.u.const_eval(lo)[1]
            b = self.u.const_eval(hi)[1]
            n *= b - a + 1
        return n


def lit(t, x):
    if t == "i":
        return str(int(x))
    if t == "l":
        return "True" if x else "False"
    if t == "c":
        return repr(x)
    r = repr(float(x))
    if r in ("inf", "-inf", "nan"):
        return "float(%r)" % r
    return r


class Program:
    """The subroutines of one source file translated to Python.  probes maps
    (subroutine, source line of a DO statement) -> a name under which every
    value the loop variable takes is appended to self.probe[name]."""

    def __init__(self, path, probes=None, with_main=False, stdin=(), replace=None, stubs=()):
        """replace maps a subroutine name to another source file whose
        subroutine of that name is used instead (to run a program with one
        routine taken from a sibling version of the file); stubs names
        subroutines that run as no-ops (graphics calls into a plotting
        library the image does not have, whether or not the file defines
        them)."""
        self.path = path
        self.stubs = set(stubs)
        self.input = ListInput(stdin)
        self.probes = dict(probes or {})
        self.statics = {}
        self.commons = {}
        self.units = {}
        for kind, name, args, stmts in read_units(path):
            if name in self.stubs:
                continue
            if kind == "subroutine":
                self.units[name] = Unit(name, args, stmts, self.commons)
            elif kind.startswith("function:"):
                u = Unit(name, args, stmts, self.commons, result=name)
                if kind[9:]:
                    u.var(name).typ = kind[9:]
                    u.var(name).explicit = True
                self.units[name] = u
            elif with_main:
                self.units["_main"] = Unit("_main", [], stmts, self.commons)
        for name, other in (replace or {}).items():
            found = [u for u in read_units(other) if u[0] == "subroutine" and u[1] == name]
            if len(found) != 1 or name not in self.units:
                raise ValueError("cannot replace %s from %s" % (name, other))
            kind, _, args, stmts = found[0]
            for key in list(self.commons):
                self.commons[key] = [(u, n) for u, n in self.commons[key] if u.name != name]
            self.units[name] = Unit(name, args, stmts, self.commons)
        self.layout = self._common_layout()
        src = ["import math", ""]
        for name in sorted(self.stubs):
            src.append("def F_%s(*args):\n    return None\n" % name)
        for u in self.units.values():
            src.append(Gen(u, self).function())
            src.append("")
        self.source = "\n".join(src)
        self.probe = {p: [] for p in self.probes.values()}
        self.common = {blk: [self._buffer(t, n) for t, n in members] for blk, members in self.layout.items()}
        self.static = {k: self._buffer(t, n) for k, (t, n) in self.statics.items()}
        self.ns = {"COMMON": self.common, "STATIC": self.static, "PROBE": self.probe, "INPUT": self.input, "r4": r4,
                   "idiv": idiv, "ipow": ipow, "powi": powi, "trip": trip, "nint": nint,
                   "FortranStop": FortranStop}
        exec(compile(self.source, "<f77:%s>" % path, "exec"), self.ns)

    @staticmethod
    def _buffer(t, n):
        return [0] * n if t == "i" else [False] * n if t == "l" else [""] * n if t == "c" else [0.0] * n

    def _common_layout(self):
        layout = {}
        for key, decls in self.commons.items():
            blk = key[1]
            for unit, names in decls:
                members = []
                for n in names:
                    v = unit.vars[n]
                    size = 1
                    if v.dims is not None:
                        for lo, hi in v.dims:
                            size *= unit.const_eval(hi)[1] - unit.const_eval(lo)[1] + 1
                    members.append((v.typ, size))
                if blk not in layout:
                    layout[blk] = members
                elif layout[blk] != members:
                    # units that declare a block with other shapes: kept
                    # positionally (same member count and types) at the
                    # larger sizes; right for a unit that is never run or
                    # touches only the first element of a shorter member
                    old = layout[blk]
                    if len(old) != len(members) or any(a[0] != b[0] for a, b in zip(old, members)):
                        raise NotImplementedError("COMMON /%s/ laid out differently in %s: %s vs %s"
                                                  % (blk, unit.name, members, old))
                    layout[blk] = [(a[0], max(a[1], b[1])) for a, b in zip(old, members)]
        return layout

    def sub(self, name):
        return self.ns["F_" + name]

    def common_member(self, blk, name):
        """The storage list of COMMON /blk/ member `name` (by the position the
        first declaring unit gives it)."""
        for unit, names in self.commons[("decl", blk)]:
            if name in names:
                return self.common[blk][names.index(name)]
        raise KeyError(name)


class ListInput:
    """List-directed READ * from the lines of an input deck: every READ
    starts a new record; values are separated by commas or blanks and a READ
    that needs more values goes on to the next records.  A REAL*8 value is
    the decimal correctly rounded to binary64 (d exponents read as e), a REAL
    value rounded to binary32, a character value the item without quotes."""

    def __init__(self, lines):
        self.lines = list(lines)
        self.pos = 0

    def _record(self):
        if self.pos >= len(self.lines):
            raise EOFError("input deck exhausted")
        line = self.lines[self.pos]
        self.pos += 1
        return [x for x in re.split(r"[,\s]+", line.strip()) if x]

    def read(self, types):
        vals, items = [], []
        for t in types:
            while not items:
                items = self._record()
            x = items.pop(0)
            if t == "i":
                vals.append(int(x))
            elif t == "d":
                vals.append(float(x.lower().replace("d", "e")))
            elif t == "r":
                vals.append(dec_to_r4(x.lower().replace("d", "e")))
            elif t == "c":
                vals.append(x.strip("'\""))
            else:
                raise NotImplementedError("READ of type " + t)
        return vals


def ref(buf, off=0):
    """An argument reference: (storage list, offset)."""
    return (buf, off)


def cell(value):
    return ([value], 0)
