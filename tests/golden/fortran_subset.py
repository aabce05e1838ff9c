"""Execute the reference's Fortran solver source text statement by statement.

This is a translator for the small Fortran 90 subset that the Krylov solver
files of T-FlowS use (Process/CG.f90, BiCG.f90, CGS.f90, Prec1.f90,
Resid.f90): SUBROUTINE headers, INTEGER/REAL declarations with explicit
bounds, DO loops with steps, block and one-line IF, GOTO to a label at
subroutine level, CALL (scalar actual arguments that are variables receive
the dummy's final value, as pass-by-reference does), assignments including
whole-array ones (`a = 0.0`, `a = b`) and the intrinsics
sqrt/min/max/real/abs.
Each subroutine becomes a Python function.  Real values are numpy float64
scalars: IEEE binary64 with correctly rounded + - * / and sqrt and IEEE
results for x/0 (Inf or NaN, no exception), which is what gfortran emits for
REAL*8 (-fdefault-real-8) without -ffast-math and without FMA contraction.
Sums are evaluated left to right, as Fortran and Python both do for a chain
of binary operators.

It is used only to generate the golden fixtures in this directory (see
make_golden.py); nothing at test or run time imports it.
"""
import math
import re

import numpy as np

__all__ = ["FArr", "Module", "translate", "load_subroutines"]


class _Goto(Exception):
    def __init__(self, label):
        self.label = label


class FArr:
    """A Fortran array dummy: storage list, offset of its first element and
    the lower bound the declaring scope gives it (sequence association)."""

    __slots__ = ("buf", "off", "lo")

    def __init__(self, buf, off=0, lo=1):
        self.buf, self.off, self.lo = buf, off, lo

    def __getitem__(self, i):
        return self.buf[self.off + i - self.lo]

    def __setitem__(self, i, v):
        self.buf[self.off + i - self.lo] = v

    def view(self, lo):
        return FArr(self.buf, self.off, lo)


class Module:
    """Module variables shared by the translated subroutines (sol_mod,
    par_mod and allp_mod of the reference, single-domain values)."""

    def __init__(self, **kw):
        self.__dict__.update(kw)


def _trip(a, b, s):
    n = b - a + s
    if s == 0:
        raise ValueError("zero DO step")
    q = int(n / s)
    return q if q > 0 else 0


_TOKEN = re.compile(
    r"\s*(?:(?P<num>(?:\d+\.\d*|\.\d+|\d+)(?:[eEdD][+-]?\d+)?)"
    r"|(?P<dotop>\.(?:and|or|not|lt|le|gt|ge|eq|ne|true|false)\.)"
    r"|(?P<name>[a-z_][a-z0-9_]*)"
    r"|(?P<op>\*\*|<=|>=|==|/=|[-+*/(),<>:=]))"
)

_DOTOPS = {
    ".and.": " and ", ".or.": " or ", ".not.": " not ", ".lt.": "<",
    ".le.": "<=", ".gt.": ">", ".ge.": ">=", ".eq.": "==", ".ne.": "!=",
    ".true.": "True", ".false.": "False",
}
_INTRINSICS = {"sqrt": "_sqrt", "min": "min", "max": "max", "real": "float",
               "abs": "abs", "dble": "float"}
_NOOP_CALLS = {"glosum", "exchng", "wait", "igLsum".lower(), "glomax", "glomin"}


def _tokens(s):
    pos, out = 0, []
    s = s.rstrip()
    while pos < len(s):
        m = _TOKEN.match(s, pos)
        if not m or m.end() == pos:
            raise SyntaxError(f"cannot tokenize: {s[pos:]!r}")
        pos = m.end()
        for kind in ("num", "dotop", "name", "op"):
            v = m.group(kind)
            if v is not None:
                out.append((kind, v))
                break
    return out


class _Scope:
    def __init__(self, arrays, module_names, params):
        self.arrays = arrays            # names that are arrays in this scope
        self.module_names = module_names
        self.params = params            # named constants -> python literal

    def ref(self, name):
        if name in self.params:
            return self.params[name]
        if name in self.module_names:
            return "M." + name
        return name


def _expr(toks, scope):
    out, stack = [], []
    i = 0
    while i < len(toks):
        kind, v = toks[i]
        nxt = toks[i + 1][1] if i + 1 < len(toks) else None
        if kind == "num":
            out.append(v.replace("d", "e").replace("D", "e"))
        elif kind == "dotop":
            out.append(_DOTOPS[v])
        elif kind == "name":
            if nxt == "(" and v in _INTRINSICS:
                out.append(_INTRINSICS[v] + "(")
                stack.append(")")
                i += 1
            elif nxt == "(" and v in scope.arrays:
                out.append(scope.ref(v) + "[")
                stack.append("]")
                i += 1
            elif nxt == "(":
                raise SyntaxError(f"unknown function or array {v!r}")
            else:
                out.append(scope.ref(v))
        else:
            if v == "(":
                out.append("(")
                stack.append(")")
            elif v == ")":
                out.append(stack.pop())
            elif v == "/=":
                out.append("!=")
            else:
                out.append(v)
        i += 1
    if stack:
        raise SyntaxError("unbalanced parentheses")
    return "".join(out)


def _split_top(toks, sep=","):
    parts, depth, cur = [], 0, []
    for t in toks:
        if t[1] == "(":
            depth += 1
        elif t[1] == ")":
            depth -= 1
        if t[1] == sep and depth == 0:
            parts.append(cur)
            cur = []
        else:
            cur.append(t)
    parts.append(cur)
    return parts


def _match_paren(toks, start):
    depth = 0
    for i in range(start, len(toks)):
        if toks[i][1] == "(":
            depth += 1
        elif toks[i][1] == ")":
            depth -= 1
            if depth == 0:
                return i
    raise SyntaxError("unbalanced parentheses")


def _logical_lines(text):
    lines, buf = [], ""
    for raw in text.splitlines():
        line = raw.split("!", 1)[0].rstrip()
        if not line.strip():
            continue
        if line.endswith("&"):
            buf += line[:-1] + " "
            continue
        buf += line
        if buf.lstrip().startswith("&"):
            buf = buf.lstrip()[1:]
        lines.append(buf.strip().lower())
        buf = ""
    return lines


def translate(text, module_names, params, subroutines):
    """Translate every SUBROUTINE in `text` to Python source; `subroutines`
    maps each callable subroutine name to its dummy argument names."""
    lines = _logical_lines(text)
    out = []
    i = 0
    while i < len(lines):
        m = re.match(r"subroutine\s+(\w+)\s*\((.*)\)$", lines[i])
        if not m:
            i += 1
            continue
        name = m.group(1)
        args = [a.strip() for a in m.group(2).split(",") if a.strip()]
        body = []
        i += 1
        while not re.match(r"end\s*subroutine", lines[i]) and lines[i] != "end":
            body.append(lines[i])
            i += 1
        i += 1
        out.append(_translate_sub(name, args, body, module_names, params, subroutines))
    return "\n".join(out)


def _translate_sub(name, args, body, module_names, params, subroutines):
    arrays, decl_bounds, locals_ = set(), {}, set()
    stmts = []
    for line in body:
        if line.startswith("use ") or line.startswith("implicit"):
            continue
        m = re.match(r"(integer|real)\s*(?:,[^:]*)?::(.*)$", line)
        if m:
            for part in _split_top(_tokens(m.group(2))):
                vname = part[0][1]
                if len(part) > 1:
                    arrays.add(vname)
                    close = _match_paren(part, 1)
                    dims = _split_top(part[2:close])
                    lo = "1"
                    d0 = _split_top(dims[0], ":")
                    if len(d0) == 2:
                        lo = ("lo", d0[0])
                    decl_bounds[vname] = lo
                if vname not in args:
                    locals_.add(vname)
            continue
        stmts.append(line)
    # Names declared here shadow module names of the same spelling.
    mod = set(module_names) - set(args) - locals_
    mod_arrays = {n for n in mod if n in module_names and module_names[n] == "array"}
    scope = _Scope(arrays | mod_arrays, mod, params)

    src = [f"def {name}(M, {', '.join(args)}):"]
    ind = "    "
    for a in args:
        if a in arrays:
            lo = decl_bounds[a]
            if isinstance(lo, tuple):
                src.append(f"{ind}{a} = {a}.view({_expr(lo[1], scope)})")
            else:
                src.append(f"{ind}{a} = {a}.view(1)")
    for loc in sorted(locals_ - arrays):
        src.append(f"{ind}{loc} = 0")
    has_goto = any(re.search(r"\bgo\s*to\b", s) for s in stmts)
    level = 1
    if has_goto:
        src.append(ind + "try:")
        level = 2
    loop_id = [0]
    block = []  # stack of block kinds

    def emit(s):
        src.append(ind * level + s)

    def simple(stmt):
        st = stmt.strip()
        m = re.match(r"go\s*to\s+(\d+)$", st)
        if m:
            return f"raise _Goto({m.group(1)})"
        if st == "return":
            return "return locals()"
        if st == "continue":
            return "pass"
        m = re.match(r"call\s+(\w+)\s*(?:\((.*)\))?$", st)
        if m:
            cname = m.group(1)
            if cname in _NOOP_CALLS:
                return "pass"
            if cname not in subroutines:
                raise SyntaxError(f"call to unknown subroutine {cname}")
            cargs = _split_top(_tokens(m.group(2) or ""))
            pas, back = [], []
            dummies = subroutines[cname]
            for k, ca in enumerate(cargs):
                if len(ca) == 1 and ca[0][0] == "name" and ca[0][1] in scope.arrays:
                    pas.append(scope.ref(ca[0][1]))
                else:
                    pas.append(_expr(ca, scope))
                    if (len(ca) == 1 and ca[0][0] == "name" and ca[0][1] not in scope.params
                            and k < len(dummies)):
                        back.append(f"{scope.ref(ca[0][1])} = _r[{dummies[k]!r}]")
            call = f"{cname}(M, {', '.join(pas)})"
            return "; ".join([f"_r = {call}"] + back) if back else call
        # assignment: variable or array element, '=', expression
        m = re.match(r"^([a-z_]\w*\s*(?:\([^=]*\))?)\s*=(?!=)(.*)$", st)
        if not m:
            raise SyntaxError(f"unsupported statement {st!r}")
        ltoks = _tokens(m.group(1))
        if len(ltoks) == 1 and ltoks[0][1] in scope.arrays:
            # whole-array assignment: from an array of the same shape, or a scalar
            rtoks = _tokens(m.group(2))
            lhs = scope.ref(ltoks[0][1])
            if len(rtoks) == 1 and rtoks[0][0] == "name" and rtoks[0][1] in scope.arrays:
                return f"_acopy({lhs}, {scope.ref(rtoks[0][1])})"
            return f"_afill({lhs}, {_expr(rtoks, scope)})"
        lhs = _expr(ltoks, scope)
        rhs = _expr(_tokens(m.group(2)), scope)
        return f"{lhs} = {rhs}"

    for stmt in stmts:
        lab = re.match(r"^(\d+)\s+(.*)$", stmt)
        if lab:
            if level != 2 or not has_goto:
                raise SyntaxError("labels are supported only at subroutine level")
            emit("pass")
            src.append(ind + "except _Goto:")
            src.append(ind * 2 + "pass")
            level = 1
            has_goto = False
            stmt = lab.group(2)
        m = re.match(r"do\s+(\w+)\s*=\s*(.*)$", stmt)
        if m:
            var = scope.ref(m.group(1))
            parts = _split_top(_tokens(m.group(2)))
            a = _expr(parts[0], scope)
            b = _expr(parts[1], scope)
            s = _expr(parts[2], scope) if len(parts) > 2 else "1"
            loop_id[0] += 1
            n = loop_id[0]
            emit(f"_s{n} = {s}")
            emit(f"_n{n} = _trip({a}, {b}, _s{n})")
            emit(f"{var} = {a}")
            emit(f"for _t{n} in range(_n{n}):")
            block.append(("do", var, n))
            level += 1
            continue
        if re.match(r"end\s*do$", stmt):
            kind, var, n = block.pop()
            emit(f"{var} += _s{n}")
            level -= 1
            continue
        if stmt.startswith("if") and re.match(r"if\s*\(", stmt):
            toks = _tokens(stmt)
            close = _match_paren(toks, 1)
            cond = _expr(toks[2:close], scope)
            rest = toks[close + 1:]
            if rest == [("name", "then")]:
                emit(f"if {cond}:")
                block.append(("if",))
                level += 1
                emit("pass")
            else:
                # one-line IF: the statement after the condition's ')'
                depth, k = 0, 0
                txt = stmt
                for k, ch in enumerate(txt):
                    if ch == "(":
                        depth += 1
                    elif ch == ")":
                        depth -= 1
                        if depth == 0:
                            break
                emit(f"if {cond}:")
                level += 1
                emit(simple(txt[k + 1:]))
                level -= 1
            continue
        m = re.match(r"else\s*if\s*\((.*)\)\s*then$", stmt)
        if m:
            toks = _tokens(stmt[stmt.index("("):])
            close = _match_paren(toks, 0)
            cond = _expr(toks[1:close], scope)
            level -= 1
            emit(f"elif {cond}:")
            level += 1
            emit("pass")
            continue
        if stmt == "else":
            level -= 1
            emit("else:")
            level += 1
            emit("pass")
            continue
        if re.match(r"end\s*if$", stmt):
            block.pop()
            level -= 1
            continue
        emit(simple(stmt))
    if has_goto:
        emit("pass")
        src.append(ind + "except _Goto:")
        src.append(ind * 2 + "pass")
    src.append(ind + "return locals()")
    return "\n".join(src) + "\n"


def _sqrt(x):
    return np.sqrt(np.float64(x))


def _afill(a, v):
    for k in range(a.off, len(a.buf)):
        a.buf[k] = v


def _acopy(a, b):
    n = len(a.buf) - a.off
    a.buf[a.off:] = b.buf[b.off:b.off + n]


def load_subroutines(texts, module_names, params):
    """Translate the given Fortran source texts and return {name: function}."""
    names = {}
    for t in texts:
        for line in _logical_lines(t):
            m = re.match(r"subroutine\s+(\w+)\s*\((.*)\)$", line)
            if m:
                names[m.group(1)] = [a.strip() for a in m.group(2).split(",") if a.strip()]
    src = "\n".join(translate(t, module_names, params, names) for t in texts)
    env = {"_Goto": _Goto, "_trip": _trip, "_sqrt": _sqrt, "math": math,
           "float": np.float64, "_afill": _afill, "_acopy": _acopy}
    exec(compile(src, "<fortran_subset>", "exec"), env)
    return {n: env[n] for n in names}, src
