"""Generate golden vectors by executing the reference's own Julia source.

Julia is not available here, so this script transliterates the reference
scripts mechanically instead of restating them by hand:

* every ``macro NAME(ix,iy,iz) esc(:( ... )) end`` is expanded textually
  (``$ix`` -> the call's argument), recursively;
* every ``@parallel_indices (ix,iy,iz) function`` / ``@parallel function`` body
  is parsed into its ``if (...) A[...] = ... end`` statements and evaluated with
  numpy over the launch range ParallelStencil infers (the per-dimension maximum
  size of the array arguments), statement by statement (the kernels are
  race-free, so this equals the GPU/Threads semantics);
* ParallelStencil.FiniteDifferences3D macros (``@all @inn @d_xa @d_xi @av_xa
  @av_xi @av_xyi @av_xya @maxloc`` ...) are expanded by their published
  definitions (ParallelStencil.jl; version unpinned, the reference ships no
  Manifest.toml);
* the body of the solver function is executed line by line: parameter and
  preprocessing assignments, ``@zeros/@ones`` allocations, the ``@parallel``
  initialisation calls, then the PT loop body (``@parallel`` calls, helper
  functions such as ``copy_BC!``, and scalar ``if`` blocks) for k iterations.

Grid sizes are overridden (small grids); everything else comes from the
source text.  Output: ``tests/golden/<case>.npz`` with the initial fields
(``in_<name>``), the fields after k iterations (``k<k>_<name>``) and the
scalars used.  Run from the repository root:

    python tests/golden/make_golden.py [/path/to/reference]
"""
from __future__ import annotations

import math
import re
import sys
from pathlib import Path

import numpy as np

OUT = Path(__file__).resolve().parent

# --------------------------------------------------------------------------
# ParallelStencil.FiniteDifferences3D (published definitions; A[ix,iy,iz] 1-based)
FD = {
    "all": "{A}[ix,iy,iz]",
    "inn": "{A}[ix+1,iy+1,iz+1]",
    "d_xa": "({A}[ix+1,iy,iz]-{A}[ix,iy,iz])",
    "d_ya": "({A}[ix,iy+1,iz]-{A}[ix,iy,iz])",
    "d_za": "({A}[ix,iy,iz+1]-{A}[ix,iy,iz])",
    "d_xi": "({A}[ix+1,iy+1,iz+1]-{A}[ix,iy+1,iz+1])",
    "d_yi": "({A}[ix+1,iy+1,iz+1]-{A}[ix+1,iy,iz+1])",
    "d_zi": "({A}[ix+1,iy+1,iz+1]-{A}[ix+1,iy+1,iz])",
    "av_xa": "(({A}[ix,iy,iz]+{A}[ix+1,iy,iz])*0.5)",
    "av_ya": "(({A}[ix,iy,iz]+{A}[ix,iy+1,iz])*0.5)",
    "av_za": "(({A}[ix,iy,iz]+{A}[ix,iy,iz+1])*0.5)",
    "av_xi": "(({A}[ix,iy+1,iz+1]+{A}[ix+1,iy+1,iz+1])*0.5)",
    "av_yi": "(({A}[ix+1,iy,iz+1]+{A}[ix+1,iy+1,iz+1])*0.5)",
    "av_zi": "(({A}[ix+1,iy+1,iz]+{A}[ix+1,iy+1,iz+1])*0.5)",
    "av_xyi": "(({A}[ix,iy,iz+1]+{A}[ix+1,iy,iz+1]+{A}[ix,iy+1,iz+1]+{A}[ix+1,iy+1,iz+1])*0.25)",
    "av_xzi": "(({A}[ix,iy+1,iz]+{A}[ix+1,iy+1,iz]+{A}[ix,iy+1,iz+1]+{A}[ix+1,iy+1,iz+1])*0.25)",
    "av_yzi": "(({A}[ix+1,iy,iz]+{A}[ix+1,iy+1,iz]+{A}[ix+1,iy,iz+1]+{A}[ix+1,iy+1,iz+1])*0.25)",
    "av_xya": "(({A}[ix,iy,iz]+{A}[ix+1,iy,iz]+{A}[ix,iy+1,iz]+{A}[ix+1,iy+1,iz])*0.25)",
    "av_xza": "(({A}[ix,iy,iz]+{A}[ix+1,iy,iz]+{A}[ix,iy,iz+1]+{A}[ix+1,iy,iz+1])*0.25)",
    "av_yza": "(({A}[ix,iy,iz]+{A}[ix,iy+1,iz]+{A}[ix,iy,iz+1]+{A}[ix,iy+1,iz+1])*0.25)",
    "maxloc": ("max(max(max(max({A}[ix,iy+1,iz+1],{A}[ix+2,iy+1,iz+1]),{A}[ix+1,iy+1,iz+1]),"
               "max({A}[ix+1,iy,iz+1],{A}[ix+1,iy+2,iz+1])),max({A}[ix+1,iy+1,iz],{A}[ix+1,iy+1,iz+2]))"),
}


def strip_comments(src: str) -> str:
    out = []
    for line in src.splitlines():
        q = False
        for i, ch in enumerate(line):
            if ch == '"':
                q = not q
            if ch == "#" and not q:
                line = line[:i]
                break
        out.append(line)
    return "\n".join(out)


def match_paren(s: str, i: int) -> int:
    """index of the bracket closing s[i] (one of ( [)."""
    pairs = {"(": ")", "[": "]"}
    stack = [pairs[s[i]]]
    j = i + 1
    while stack:
        ch = s[j]
        if ch in pairs:
            stack.append(pairs[ch])
        elif ch in ")]":
            if ch != stack[-1]:
                raise ValueError("unbalanced brackets")
            stack.pop()
        j += 1
    return j - 1


def split_args(s: str) -> list[str]:
    args, depth, cur = [], 0, ""
    for ch in s:
        if ch in "([":
            depth += 1
        elif ch in ")]":
            depth -= 1
        if ch == "," and depth == 0:
            args.append(cur.strip())
            cur = ""
        else:
            cur += ch
    if cur.strip():
        args.append(cur.strip())
    return args


IDENT = r"[^\W\d][\w!]*"


class Script:
    def __init__(self, path: Path):
        self.src = strip_comments(path.read_text())
        self.macros = self._macros()
        self.kernels = self._kernels()
        self.functions = self._plain_functions()

    # -- macros -----------------------------------------------------------------
    def _macros(self) -> dict:
        res = {}
        for m in re.finditer(r"macro\s+(" + IDENT + r")\s*\(([^)]*)\)\s*esc\(:\(", self.src):
            start = m.end() - 1
            end = match_paren(self.src, start)
            res[m.group(1)] = ([a.strip() for a in m.group(2).split(",")], self.src[start + 1:end])
        return res

    def expand(self, expr: str) -> str:
        for _ in range(50):
            m = None
            for mm in re.finditer(r"@(" + IDENT + r")\s*\(", expr):
                if mm.group(1) in self.macros or mm.group(1) in FD:
                    m = mm
                    break
            if m is None:
                return expr
            name = m.group(1)
            o = m.end() - 1
            c = match_paren(expr, o)
            args = split_args(expr[o + 1:c])
            if name in self.macros:
                params, body = self.macros[name]
                for p_, a in zip(params, args):
                    body = re.sub(r"\$" + re.escape(p_) + r"(?![\w])", "(" + a + ")", body)
                rep = "(" + body + ")"
            else:
                rep = FD[name].format(A=args[0])
            expr = expr[:m.start()] + rep + expr[c + 1:]
        raise RuntimeError("macro expansion did not terminate")

    # -- kernels -------------------------------------------------------------------
    def _kernels(self) -> dict:
        res = {}
        for m in re.finditer(r"@parallel(_indices\s*\((\w+),(\w+),(\w+)\))?\s+function\s+(" + IDENT + r")\s*\(", self.src):
            name = m.group(5)
            o = m.end() - 1
            c = match_paren(self.src, o)
            params = [_rename(a.split("::")[0].strip()) for a in split_args(self.src[o + 1:c])]
            body, _ = self._block(self.src, c + 1)
            res[name] = {"params": params, "fd": m.group(1) is None, "body": body}
        return res

    def _plain_functions(self) -> dict:
        """helper functions made only of @parallel calls (e.g. copy_BC!)"""
        res = {}
        for m in re.finditer(r"(?<!@parallel )(?<!_indices \(ix,iy,iz\) )\nfunction\s+(" + IDENT + r")\s*\(", self.src):
            o = m.end() - 1
            c = match_paren(self.src, o)
            params = [a.split("::")[0].strip() for a in split_args(self.src[o + 1:c])]
            body, _ = self._block(self.src, c + 1)
            calls = re.findall(r"@parallel\s+(" + IDENT + r")\(([^)]*)\)", " ".join(_flatten_text(body)))
            if calls:
                res[m.group(1)] = {"params": params, "calls": calls}
        return res

    _OPENERS = {"if", "function", "for", "while", "begin", "let"}

    def _block(self, s: str, i: int):
        """statements from i to the matching `end`; returns (statements, index after end)."""
        stmts = []
        n = len(s)
        while i < n:
            while i < n and s[i] in " \t\n;":
                i += 1
            m = re.match(r"(" + IDENT + r")", s[i:])
            word = m.group(1) if m else ""
            if word == "end":
                return stmts, i + 3
            if word == "return":
                i += 6
                continue
            if word == "if":
                j = i + 2
                while s[j] in " \t":
                    j += 1
                if s[j] != "(":
                    raise ValueError("unparenthesised if condition")
                c = match_paren(s, j)
                cond = s[j + 1:c]
                body, i = self._block(s, c + 1)
                stmts.append(("if", cond, body))
                continue
            # assignment statement: up to a depth-0 newline without continuation, or `end`
            j, depth = i, 0
            while j < n:
                ch = s[j]
                if ch in "([":
                    depth += 1
                elif ch in ")]":
                    depth -= 1
                elif depth == 0 and ch == "\n":
                    prev = s[i:j].rstrip()
                    if not re.search(r"([+\-*/^=,&|]|&&|\|\|)$", prev):
                        break
                elif depth == 0 and re.match(r"\bend\b", s[j:]) and not re.match(r"\w", s[j - 1]):
                    break
                j += 1
            stmts.append(("set", s[i:j].strip()))
            i = j
        raise ValueError("unterminated block")


def _flatten_text(body):
    for st in body:
        if st[0] == "set":
            yield st[1]
        else:
            yield from _flatten_text(st[2])


# --------------------------------------------------------------------------
# Julia expression -> Python/numpy
PY_KEYWORDS = {"in", "is", "lambda", "not", "and", "or", "from", "global", "pass", "def", "class", "del", "yield", "as", "with"}


def _rename(e: str) -> str:
    """Julia identifiers that are Python keywords get a trailing underscore"""
    return re.sub(r"(?<![\w.])(" + "|".join(sorted(PY_KEYWORDS)) + r")(?![\w])", r"\1_", e)


def py_expr(e: str) -> str:
    e = _rename(e).replace("\n", " ")
    e = e.replace("&&", " & ").replace("||", " | ").replace("^", "**").replace("π", "pi")
    # array indexing NAME[a,b,c] -> G(NAME, a, b, c)
    out, i = "", 0
    while i < len(e):
        m = re.match(r"(" + IDENT + r")\[", e[i:])
        if m and (i == 0 or not re.match(r"[\w.]", e[i - 1])):
            name = m.group(1)
            o = i + m.end() - 1
            c = match_paren(e, o)
            args = split_args(e[o + 1:c])
            out += "G(" + name + "," + ",".join(py_expr(a) for a in args) + ")"
            i = c + 1
        else:
            out += e[i]
            i += 1
    return out


def py_cond(e: str) -> str:
    # wrap each &&-term in parentheses (Python's & binds tighter than comparisons)
    parts, depth, cur = [], 0, ""
    k = 0
    while k < len(e):
        if e[k] in "([":
            depth += 1
        elif e[k] in ")]":
            depth -= 1
        if depth == 0 and e.startswith("&&", k):
            parts.append(cur)
            cur = ""
            k += 2
            continue
        cur += e[k]
        k += 1
    parts.append(cur)
    return " & ".join("(" + py_expr(p) + ")" for p in parts)


def G(A, i, j, k):
    i, j, k = (np.asarray(x) for x in (i, j, k))
    if (np.any(i < 1) or np.any(j < 1) or np.any(k < 1) or np.any(i > A.shape[0]) or np.any(j > A.shape[1])
            or np.any(k > A.shape[2])):
        raise IndexError("out-of-range read in the transliterated kernel")
    return A[i - 1, j - 1, k - 1]


def _max(*a):
    out = a[0]
    for x in a[1:]:
        out = np.maximum(out, x)
    return out


def _min(*a):
    out = a[0]
    for x in a[1:]:
        out = np.minimum(out, x)
    return out


MATH = {"G": G, "pi": math.pi, "sin": np.sin, "cos": np.cos, "cot": lambda x: 1.0 / np.tan(x), "sqrt": np.sqrt,
        "exp": np.exp, "log": np.log, "abs": np.abs, "max": _max, "min": _min, "log10": math.log10,
        "size": lambda A, d: A.shape[d - 1], "mod": lambda a, b: a % b}


class Runner:
    def __init__(self, script: Script, env: dict):
        self.s = script
        self.env = env
        self.cache = {}

    def _compile(self, text: str, mode="eval"):
        key = (text, mode)
        if key not in self.cache:
            self.cache[key] = compile(text.strip(), "<jl>", mode)
        return self.cache[key]

    def kernel(self, name: str, args: list[str]):
        k = self.s.kernels[name]
        loc = dict(MATH)
        arrays = []
        for p_, a in zip(k["params"], args):
            v = eval(self._compile(py_expr(a)), MATH, self.env)
            loc[p_] = v
            if isinstance(v, np.ndarray):
                arrays.append(v)
        rng = [max(a.shape[d] for a in arrays) for d in range(3)]
        ix, iy, iz = np.meshgrid(*(np.arange(1, n + 1) for n in rng), indexing="ij")
        pts = (ix.ravel(), iy.ravel(), iz.ravel())
        body = k["body"]
        if k["fd"]:
            body = [self._fd_stmt(st) for st in body]
        self._exec(body, loc, pts)

    def _fd_stmt(self, st):
        m = re.match(r"@(all|inn)\((" + IDENT + r")\)\s*=\s*(.*)$", st[1], flags=re.S)
        A, rhs = m.group(2), m.group(3)
        if m.group(1) == "all":
            return ("if", f"ix<=size({A},1) && iy<=size({A},2) && iz<=size({A},3)", [("set", f"{A}[ix,iy,iz] = {rhs}")])
        return ("if", f"ix<=size({A},1)-2 && iy<=size({A},2)-2 && iz<=size({A},3)-2", [("set", f"{A}[ix+1,iy+1,iz+1] = {rhs}")])

    def _exec(self, body, loc, pts):
        for st in body:
            loc["ix"], loc["iy"], loc["iz"] = pts
            if st[0] == "if":
                mask = eval(self._compile(py_cond(self.s.expand(st[1]))), MATH, loc)
                mask = np.broadcast_to(np.asarray(mask, dtype=bool), pts[0].shape)
                if mask.any():
                    self._exec(st[2], loc, tuple(p_[mask] for p_ in pts))
            else:
                lhs, rhs = st[1].split("=", 1)
                lhs = lhs.strip()
                m = re.match(r"(" + IDENT + r")\[(.*)\]$", lhs, flags=re.S)
                A = loc[m.group(1)]
                idx = [eval(self._compile(py_expr(self.s.expand(a))), MATH, loc) for a in split_args(m.group(2))]
                val = eval(self._compile(py_expr(self.s.expand(rhs))), MATH, loc)
                idx = [np.broadcast_to(np.asarray(x), pts[0].shape) for x in idx]
                A[idx[0] - 1, idx[1] - 1, idx[2] - 1] = np.broadcast_to(val, pts[0].shape)

    def call(self, name: str, args: list[str]):
        if name in self.s.kernels:
            self.kernel(name, args)
        elif name in self.s.functions:
            f = self.s.functions[name]
            sub = dict(zip(f["params"], args))
            for kname, kargs in f["calls"]:
                self.kernel(kname, [sub.get(a.strip(), a.strip()) for a in split_args(kargs)])
        else:
            raise KeyError(name)

    def run_lines(self, lines: list[str]):
        """execute a list of script lines: @parallel calls, helper calls, assignments, scalar ifs"""
        i = 0
        while i < len(lines):
            ln = lines[i].strip()
            i += 1
            if not ln or ln.startswith(("print", "@printf", "push!", "display", "println")):
                continue
            m = re.match(r"@parallel\s+(" + IDENT + r")\((.*)\)\s*$", ln)
            if m:
                self.call(m.group(1), split_args(m.group(2)))
                continue
            m = re.match(r"(" + IDENT + r")\((.*)\)\s*$", ln)
            if m and m.group(1) in self.s.functions:
                self.call(m.group(1), split_args(m.group(2)))
                continue
            if re.match(r"if\b", ln):
                if re.match(r"if\s*\(", ln):
                    o = ln.index("(")
                    c = match_paren(ln, o)
                    cond, rest = ln[o + 1:c], ln[c + 1:].strip()
                else:
                    cond, rest = ln[2:].strip(), ""
                if re.search(r"\bend$", rest):  # one-line `if (cond) a; b end`
                    body = [x.strip() for x in re.sub(r"\bend$", "", rest).split(";") if x.strip()]
                else:
                    body = [rest] if rest else []
                    depth = 1
                    while True:
                        l2 = lines[i].strip()
                        i += 1
                        if re.match(r"(if|for)\b", l2) and not re.search(r"\bend\s*$", l2):
                            depth += 1
                        if l2 == "end":
                            depth -= 1
                            if depth == 0:
                                break
                        body.append(l2)
                body = [x for x in body if not x.startswith(("GC.", "break")) and "Base.time" not in x]
                # convergence-check blocks (`iter % nout == 0`) only read the state; they are not replayed
                if "nout" not in cond and eval(self._compile(py_cond(cond)), MATH, self.env):
                    self.run_lines(body)
                continue
            m = re.match(r"(" + IDENT + r")\s*\.=\s*(" + IDENT + r")$", ln)
            if m:
                self.env[m.group(1)][...] = self.env[m.group(2)]
                continue
            self.assign(ln)

    def assign(self, ln: str):
        ln = re.sub(r"\brange\(([^()]*(?:\([^()]*\)[^()]*)*?),\s*length\s*=\s*([^()]+)\)", r"_range(\1, \2)", ln)
        ln = ln.replace("@zeros(", "_zeros(").replace("@ones(", "_ones(")
        m = re.match(r"\(\s*(" + IDENT + r"(?:\s*,\s*" + IDENT + r")*)\s*\)\s*=\s*\((.*)\)$", ln)
        if m and " for " in m.group(2):  # coordinate comprehensions
            names = [n.strip() for n in m.group(1).split(",")]
            comps = split_args(m.group(2))
            for nm, comp in zip(names, comps):
                cm = re.match(r"\[\s*(\w+)\s+for\s+xc\s*=\s*(\w+)\s*,\s*yc\s*=\s*(\w+)\s*,\s*zc\s*=\s*(\w+)\s*\]", comp)
                var, a, b, c = cm.groups()
                xa, ya, za = self.env[a], self.env[b], self.env[c]
                shape = (len(xa), len(ya), len(za))
                src = {"xc": xa[:, None, None], "yc": ya[None, :, None], "zc": za[None, None, :]}[var]
                self.env[nm] = np.asfortranarray(np.broadcast_to(src, shape).astype(np.float64))
            return
        if "Data.Array(" in ln or "mkdir" in ln or "GC." in ln:
            return
        lhs, rhs = ln.split("=", 1)
        names = [n.strip() for n in lhs.split(",")]
        if any(n in self.env.get("_fixed", ()) for n in names):
            return
        val = eval(self._compile(py_expr(rhs.strip())), dict(MATH, _range=_range, _zeros=_zeros, _ones=_ones), self.env)
        if len(names) == 1:
            self.env[names[0]] = val
        else:
            for n, v in zip(names, val):
                self.env[n] = v


def _range(a, b, n):
    n = int(n)
    x = np.array([a + (b - a) * i / (n - 1) for i in range(n)], dtype=np.float64)
    x[-1] = b
    return x


def _zeros(*s):
    return np.zeros(tuple(int(x) for x in s), dtype=np.float64, order="F")


def _ones(*s):
    return np.ones(tuple(int(x) for x in s), dtype=np.float64, order="F")


def function_lines(src: str, fname: str) -> tuple[list[str], list[str]]:
    """(setup lines, PT-loop body lines) of the script's solver function"""
    lines = src.splitlines()
    start = next(i for i, l in enumerate(lines) if re.search(r"function\s+" + fname + r"\(\)", l))
    loop = next(i for i in range(start, len(lines)) if re.search(r"for\s+iter\s*=\s*1:maxiter", lines[i]))
    setup = [l for l in lines[start + 1:loop] if not re.search(r"for\s+it\s*=|@elapsed", l)]
    body, depth = [], 1
    i = loop + 1
    while depth:
        l = lines[i].strip()
        i += 1
        if re.match(r"(if|for)\b", l) and not re.search(r"\bend\s*$", l):
            depth += 1
        if l == "end":
            depth -= 1
            if depth == 0:
                break
        body.append(l)
    return join_continuations(setup), join_continuations(body)


def join_continuations(lines: list[str]) -> list[str]:
    out, cur, depth = [], "", 0
    for l in lines:
        s = l.strip()
        if not s:
            continue
        cur = (cur + " " + s) if cur else s
        depth += s.count("(") + s.count("[") - s.count(")") - s.count("]")
        if depth == 0 and not re.search(r"[,+\-*/=]$", s):
            out.append(cur)
            cur = ""
    if cur:
        out.append(cur)
    return out


# --------------------------------------------------------------------------
CASES = {
    # name: (script, solver function, grid overrides, extra env, scalar overrides, arrays to save, iteration counts)
    "sph_diapir": ("scripts_diapir/SphericalStokes_diapir.jl", "SPH_3D_Inclusion", {"nr": 11, "nθ": 9, "nφ": 7},
                   {"dmp": 4.5}, {"n_exp": 3.0},
                   ["P", "VR", "Vθ", "Vφ", "τ_RR", "τ_θθ", "τ_φφ", "τ_Rθ", "τ_Rφ", "τ_θφ", "η", "η_ini", "ηSM", "DT_R", "τII", "ρ"],
                   (1, 10)),
    "sph_plateau": ("scripts_plateau/SphericalStokes_plateau.jl", "SPH_3D_Plateau", {"nr": 12, "nθ": 7, "nφ": 6},
                    {"dmp": 4.5}, {},
                    ["P", "VR", "Vθ", "Vφ", "τ_RR", "τ_θθ", "τ_φφ", "τ_Rθ", "τ_Rφ", "τ_θφ", "η", "η_ini", "ηSM", "DT_R", "τII", "ρ"],
                    (1, 10)),
    "cyl_diapir": ("scripts_diapir/CylindricalStokes_diapir.jl", "CYL_3D_Inclusion", {"nr": 11, "nθ": 9, "nz": 7},
                   {}, {},
                   ["P", "VR", "Vθ", "VZ", "τ_RR", "τ_θθ", "τ_ZZ", "τ_Rθ", "τ_RZ", "τ_θZ", "η", "η_INI", "ηSM", "DT_R", "τII", "ρ", "η_PL"],
                   (1, 10)),
    "cyl_diapir_pl": ("scripts_diapir/CylindricalStokes_diapir.jl", "CYL_3D_Inclusion", {"nr": 11, "nθ": 9, "nz": 7},
                      {}, {"n_exp": 3.0},
                      ["P", "VR", "Vθ", "VZ", "τ_RR", "τ_θθ", "τ_ZZ", "τ_Rθ", "τ_RZ", "τ_θZ", "η", "η_INI", "ηSM", "DT_R", "τII", "ρ", "η_PL"],
                      (1, 10)),
    "cart_diapir": ("scripts_diapir/CartesianStokes_diapir.jl", "CART_3D_Inclusion_Perf", {"nx": 11, "ny": 9, "nz": 7},
                    {}, {"n_exp": 3.0},
                    ["P", "VX", "VY", "VZ", "τ_XX", "τ_YY", "τ_ZZ", "τ_XY", "τ_XZ", "τ_YZ", "η", "η_INI", "ηSM", "DT_R", "τII", "ρ", "η_PL"],
                    (1, 10)),
}


def run_case(ref: Path, name: str):
    rel, fname, grid, extra, scal, save, ks = CASES[name]
    sc = Script(ref / rel)
    setup, body = function_lines(sc.src, fname)
    env = dict(grid)
    env.update(extra)
    env["_fixed"] = set(grid) | set(scal)
    env.update(scal)
    r = Runner(sc, env)
    # setup: everything before the PT loop (parameters, grid, allocation, initialisation)
    env["it"] = 1
    setup = [ln for ln in setup if not (re.match(r"(num|runtime|err_evo|iters|t_tic|ittot)\b", ln) or ln.startswith(("print", "println")))]
    r.run_lines(setup)
    env["err"] = env.get("err", 1.0)
    data = {f"in_{a}": env[a].copy() for a in save}
    for k_, v_ in env.items():  # 1D node coordinates (range(...) results)
        if isinstance(v_, np.ndarray) and v_.ndim == 1:
            data[f"coord_{k_}"] = v_.copy()
    scalars = {k: float(v) for k, v in env.items() if isinstance(v, (int, float)) and not k.startswith("_")}
    done = 0
    for k in ks:
        while done < k:
            done += 1
            env["iter"] = done
            env["it"] = 1
            r.run_lines(body)
        for a in save:
            data[f"k{k}_{a}"] = env[a].copy()
    data["scalars_json"] = np.array(repr(scalars))
    data["script"] = np.array(rel)
    np.savez_compressed(OUT / f"{name}.npz", **data)
    print(f"{name}: {len(data)} arrays, scalars {sorted(scalars)}")


def main():
    if len(sys.argv) < 2:
        sys.exit("usage: make_golden.py <path of the SphericalStokes checkout> [case ...]")
    ref = Path(sys.argv[1])
    names = sys.argv[2:] or list(CASES)
    for n in names:
        run_case(ref, n)


if __name__ == "__main__":
    main()
