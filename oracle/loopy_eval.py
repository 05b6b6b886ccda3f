"""A small interpreter for the loopy instruction text of the reference's rate
kernels (test infrastructure only).

The reference writes each of its species-rate sub-kernels as loopy
instruction text (pyjac/core/rate_subs.py: get_plog_arrhenius_rates
:2084-2250, get_cheb_arrhenius_rates :1904-2083, get_sri_kernel
:2472-2588, get_troe_kernel :2350-2471, get_extra_var_rates :798-960, ...),
which loopy would compile.  loopy is not available here, but the text itself
is a plain imperative program for one state `j` and one loop index (the
kernel's `var_name`, usually `i`).  run() executes it in Python, one scalar
double operation at a time (IEEE binary64, as the generated C code), so the
reference's own formulas yield golden values for the forms that no shipped
kernel covers.

Supported: `<>` temporaries, assignments (also to array elements),
`if cond` / `else` / `end`, `for k` over an extra iname with its
'lo <= k < hi' domain, `#` comments, `\\` continuations, `{id=...}` options
(ignored: the text is executed in program order, which satisfies its
dependencies), the C functions exp, log, log10, exp10, pow, fmin, fmax, fabs,
fast_powi, and `0.0d`-style literals.
"""
import math
import re

import numpy as np

_OPTS = re.compile(r"\{[^{}]*\}", re.S)
_MOCK = re.compile(r"<MagicMock[^>]*>")
_LIT_D = re.compile(r"(\d)d\b")


def _fast_powi(x, n):
    n = int(n)
    if n < 0:
        x = 1.0 / x
        n = -n
    r = 1.0
    for _ in range(n):
        r = r * x
    return r


FUNCS = {
    "exp": math.exp, "log": math.log, "log10": math.log10, "exp10": lambda x: 10.0 ** x,
    "pow": math.pow, "fmin": lambda a, b: float(np.fmin(a, b)), "fmax": lambda a, b: float(np.fmax(a, b)),
    "fabs": math.fabs, "fast_powi": _fast_powi, "abs": abs,
}


def _domains(extra_inames):
    out = {}
    for name, dom in extra_inames or []:
        m = re.match(r"\s*(-?\d+)\s*<=\s*(\w+)\s*<\s*(-?\d+)\s*$", dom)
        if not m or m.group(2) != name:
            raise ValueError("unsupported iname domain %r" % dom)
        out[name] = (int(m.group(1)), int(m.group(3)))
    return out


def translate(text, extra_inames=(), unknown_index="__out__"):
    """Python source of the instruction text.  Indices loopy would take from
    a map that this environment cannot build are named `unknown_index`."""
    dom = _domains(extra_inames)
    text = _MOCK.sub(unknown_index, text)
    text = text.replace("\\\n", " ")
    lines = []
    for raw in _OPTS.sub("", text).split("\n"):
        line = raw.split("#", 1)[0].strip()
        if line:
            lines.append(line)
    out, depth = [], 0
    for line in lines:
        line = _LIT_D.sub(r"\1", line)
        if line == "end":
            depth -= 1
            continue
        if line == "else":
            out.append("    " * (depth - 1) + "else:")
            continue
        m = re.match(r"for\s+(\w+)$", line)
        if m:
            lo, hi = dom[m.group(1)]
            out.append("    " * depth + "for %s in range(%d, %d):" % (m.group(1), lo, hi))
            depth += 1
            continue
        m = re.match(r"if\s+(.*)$", line)
        if m:
            out.append("    " * depth + "if %s:" % m.group(1))
            depth += 1
            continue
        if line.startswith("<>"):
            line = line[2:].strip()
        out.append("    " * depth + line)
    if depth != 0:
        raise ValueError("unbalanced if/for/end in the instruction text")
    return "\n".join(out)


def _declared_first(pre):
    """Pre-instructions in an executable order: the declarations of
    precomputed temporaries (`<>`) before the statements that use them
    (loopy orders them by their dependencies, the generators list them in
    any order)."""
    pre = list(pre)
    return [p for p in pre if p.strip().startswith("<>")] + \
        [p for p in pre if not p.strip().startswith("<>")]


def run(knl, env, n_loop):
    """Execute a kernel of the reference for one state: its pre-instructions,
    the instructions for each value 0 .. n_loop - 1 of its loop index
    (knl.var_name), then its post-instructions.  env binds the arrays (as
    the text indexes them), the state index j and the kernel's scalar
    parameters; returns the namespace after the run."""
    ns = dict(FUNCS)
    ns.update(getattr(knl, "parameters", None) or {})
    ns.update(env)
    extra = getattr(knl, "extra_inames", None) or []
    # an output index loopy would map (a reaction of this kind -> its place
    # among all reactions) stays the kernel's own loop index here
    ui = knl.var_name
    pre = "\n".join(translate(t, extra, ui) for t in _declared_first(knl.pre_instructions or []))
    body = translate(knl.instructions, extra, ui)
    post = "\n".join(translate(t, extra, ui) for t in (getattr(knl, "post_instructions", None) or []))
    src = pre + "\nfor %s in range(%d):\n" % (knl.var_name, n_loop)
    src += "\n".join("    " + ln for ln in body.split("\n")) + "\n" if body.strip() else "    pass\n"
    src += post
    exec(compile(src, "<loopy instructions>", "exec"), ns)
    return ns
