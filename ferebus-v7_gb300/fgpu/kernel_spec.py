"""Kernel expression -> flat postfix kernel spec (the C-ABI's ``kspec``).

Host-side mirror of the reference's kernel-expression interpreter
(src/interpreter/parser.f90:100-200, src/interpreter/ast.f90:173-271):

* ``+`` is left-associative, ``*`` is right-recursive (``term`` calls itself
  after a ``*``, parser.f90 ``term``), ``*`` binds tighter than ``+``;
* parentheses group; a unary ``+`` is transparent;
* ``-`` and ``/`` parse but are rejected ("not yet implemented" in the
  reference, ast.f90:182-189);
* a number becomes a constant kernel whose value is one hyperparameter
  (ast.f90:257-271);
* a name resolves to a configured kernel: rbf, periodic, rbf-cyclic or
  linear (ast.f90:228-247).  When ``active_dimensions`` is not configured
  the kernel is active on every feature (src/config/kernel/kernel_type_config.f90:54-73).

Spec encoding (int32): a leaf is ``[op, n_active, dim_1..dim_n]`` with
1-based feature indices; an operator is ``[op]``.  Leaves appear in the same
left-to-right order as the reference's parameter vector
(src/kernels/kernel_module.f90:235-245).
"""
from __future__ import annotations

import re

RBF, PERIODIC, RBF_CYCLIC, LINEAR, CONSTANT = 1, 2, 3, 4, 5
SUM, PROD = 10, 11
LEAF_OPS = (RBF, PERIODIC, RBF_CYCLIC, LINEAR, CONSTANT)
TYPE_CODES = {"rbf": RBF, "periodic": PERIODIC, "rbf-cyclic": RBF_CYCLIC,
              "rbf_cyclic": RBF_CYCLIC, "linear": LINEAR}

_TOKEN = re.compile(r"\s*(?:(\d+\.\d*|\.\d+|\d+)|([A-Za-z_][A-Za-z0-9_\-]*)|(.))")


class KernelSpecError(ValueError):
    pass


def _tokens(text):
    pos, out = 0, []
    text = text.strip()
    while pos < len(text):
        m = _TOKEN.match(text, pos)
        if not m:
            raise KernelSpecError(f"cannot tokenise {text[pos:]!r}")
        num, name, sym = m.groups()
        if num is not None:
            out.append(("num", float(num)))
        elif name is not None:
            out.append(("id", name))
        elif sym is not None and not sym.isspace():
            if sym not in "+-*/()":
                raise KernelSpecError(f"invalid symbol {sym!r}")
            out.append((sym, sym))
        pos = m.end()
    out.append(("eof", None))
    return out


class _Parser:
    def __init__(self, text):
        self.toks = _tokens(text)
        self.i = 0

    def peek(self):
        return self.toks[self.i][0]

    def eat(self, kind):
        if self.peek() != kind:
            raise KernelSpecError(f"Invalid Syntax: expected {kind}, got {self.peek()}")
        tok = self.toks[self.i]
        self.i += 1
        return tok

    def factor(self):
        k = self.peek()
        if k == "+":
            self.eat("+")
            return self.factor()
        if k == "-":
            raise KernelSpecError("kernel minus not yet implemented")
        if k == "num":
            return ("num", self.eat("num")[1])
        if k == "(":
            self.eat("(")
            node = self.expr()
            self.eat(")")
            return node
        return ("var", self.eat("id")[1])

    def term(self):
        node = self.factor()
        while self.peek() in ("*", "/"):
            op = self.eat(self.peek())[0]
            if op == "/":
                raise KernelSpecError("kernel divide not yet implemented")
            node = ("*", node, self.term())
        return node

    def expr(self):
        node = self.term()
        while self.peek() in ("+", "-"):
            op = self.eat(self.peek())[0]
            if op == "-":
                raise KernelSpecError("kernel minus not yet implemented")
            node = ("+", node, self.term())
        return node

    def parse(self):
        node = self.expr()
        self.eat("eof")
        return node


def parse_expression(text):
    """Parse a kernel expression into a nested tuple tree."""
    return _Parser(text).parse()


def build_kspec(expression, kernels, nfeats):
    """Flatten ``expression`` into the postfix spec.

    ``kernels`` maps a kernel name to ``{"type": "rbf"|"periodic"|"rbf-cyclic"|"linear",
    "active_dimensions": [1-based dims] (optional)}``.
    Returns ``(kspec, constants)`` where ``constants`` lists the numbers that
    became constant kernels, in parameter order (their initial values).
    """
    spec, consts = [], []

    def walk(node):
        if node[0] == "num":
            spec.extend([CONSTANT, 0])
            consts.append(node[1])
        elif node[0] == "var":
            name = node[1]
            if name not in kernels:
                raise KernelSpecError(f"unknown kernel {name!r}")
            cfg = kernels[name]
            code = TYPE_CODES.get(str(cfg.get("type", "")).lower())
            if code is None:
                raise KernelSpecError(f"unsupported kernel type {cfg.get('type')!r}")
            dims = list(cfg.get("active_dimensions") or range(1, nfeats + 1))
            for d in dims:
                if not 1 <= int(d) <= nfeats:
                    raise KernelSpecError(f"active dimension {d} outside 1..{nfeats}")
            spec.extend([code, len(dims)] + [int(d) for d in dims])
        else:
            walk(node[1])
            walk(node[2])
            spec.append(SUM if node[0] == "+" else PROD)

    walk(parse_expression(expression))
    return spec, consts


def parse_kspec(kspec):
    """Split a postfix spec into nodes: ``("leaf", op, dims0)`` / ``("op", op)``."""
    nodes, i, ks = [], 0, [int(v) for v in kspec]
    depth = 0
    while i < len(ks):
        op = ks[i]
        if op in LEAF_OPS:
            if i + 1 >= len(ks):
                raise KernelSpecError("truncated leaf")
            n = ks[i + 1]
            if n < 0 or i + 2 + n > len(ks):
                raise KernelSpecError("bad leaf length")
            nodes.append(("leaf", op, [d - 1 for d in ks[i + 2:i + 2 + n]]))
            i += 2 + n
            depth += 1
        elif op in (SUM, PROD):
            if depth < 2:
                raise KernelSpecError("operator without two operands")
            nodes.append(("op", op))
            i += 1
            depth -= 1
        else:
            raise KernelSpecError(f"bad opcode {op}")
    if depth != 1:
        raise KernelSpecError("spec does not reduce to one kernel")
    return nodes


def nparams(kspec):
    """Kernel hyperparameter count (``Kernel%nparams``)."""
    return sum(1 if n[1] == CONSTANT else len(n[2]) for n in parse_kspec(kspec) if n[0] == "leaf")
