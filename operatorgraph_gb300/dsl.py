"""Front end for grammars written in the reference's .pga language.

The reference compiles .pga files (src/compiler: Parser.cpp, DispatchTableGenerator.cpp)
into dispatch tables that its interpreter runs with a generic procedure list
(src/interpreter/PGAFacade.cu).  This module does the same for the GB300 engine:
`parse(text)` builds a syntax tree for the language as the reference's grammars
use it, and `lower(grammar)` turns it into a dispatch table on the engine's
generic procedure list (grammar.DEFAULT_PROCS) plus the axiom shape and entry.

The language:

    axiom Box A;                          // root shape and rule
    terminal B (1, 0);                    // name(s), (generation function, terminal index)
    A = IfSizeLess(X, 0.111) { B | SubX };
    SubX = SubDiv(X) { -1: SubY | -1: Discard() | -1: SubY };
    F = Extrude(Exp(ShapeSize(X) * 0.5)) Repeat(Y, 3, ANCHOR_TO_START) Tile;

A rule body is a chain of operators; a branching operator ends it with a
`{ a | b | ... }` block (SubDiv and RandomRule successors carry `factor:`), any other
operator passes its shape to what follows; a chain ends in a rule name, a
terminal name, `Discard()` or a block.  Arguments are numbers, axes X/Y/Z,
repeat modes, ShapeSize / ShapeNormal / ShapePos / ShapeSeed /
ShapeCustomAttribute, Rand(min, max) and Exp(infix expression).

Lowered operators, with the reference generator's parameter layouts
(DispatchTableGenerator.cpp:266-440, 541-554): SubDiv (axis, factors...) as
the dynamic Subdivide, Repeat (axis, extent, mode), CompSplit (successors top,
bottom, sides), Extrude (axis slot, extent), IfSizeLess (axis, size; true,
false), If (condition; true, false), Translate (x, y, z), Scale (x, y, z),
Rotate (x, y, z degrees), SwapSize (three axes), RandomRule (chance,
weights...; one successor per weight), Replicate (successors), Discard, and
terminals as Generate (terminal index; generation function 1 is the instanced
one, 0 the triangle mesh that pga_generate_meshes expands).  The others (the
prism SetAs operators, IfCollides...) parse but are not engine operators:
lowering raises DslError naming the operator and the rule.  A rule applied to both a Box and a
Quad is lowered once per shape.
"""
import re

import numpy as np

from . import grammar as G

AXES = {"X": 0, "Y": 1, "Z": 2}
MODES = {"ANCHOR_TO_START": G.ANCHOR_TO_START, "ANCHOR_TO_END": G.ANCHOR_TO_END,
         "ADJUST_TO_FILL": G.ADJUST_TO_FILL}
SHAPES = {"Box": G.SHAPE_BOX, "Quad": G.SHAPE_QUAD}
BRANCHING = {"SubDiv", "CompSplit", "IfSizeLess", "If", "Replicate", "RandomRule"}
SUPPORTED = {"SubDiv", "Repeat", "CompSplit", "Extrude", "IfSizeLess", "Discard", "Translate", "Scale", "RandomRule",
             "Rotate", "Replicate", "If", "SwapSize"}


class DslError(ValueError):
    pass


# ------------------------------------------------------------------ tokenizer

_TOKEN = re.compile(r"""
    (?P<ws>\s+|//[^\n]*|/\*.*?\*/)
  | (?P<num>(?:\d+\.\d*|\.\d+|\d+)(?:[eE][-+]?\d+)?)
  | (?P<name>[A-Za-z_][A-Za-z_0-9]*)
  | (?P<op>==|!=|<=|>=|&&|\|\||[-+*/<>(){}|:;,=])
""", re.S | re.X)


def tokenize(text):
    out, pos = [], 0
    while pos < len(text):
        m = _TOKEN.match(text, pos)
        if not m:
            line = text.count("\n", 0, pos) + 1
            raise DslError(f"line {line}: unexpected character {text[pos]!r}")
        pos = m.end()
        if m.lastgroup == "ws":
            continue
        line = text.count("\n", 0, m.start()) + 1
        out.append((m.lastgroup, m.group(), line))
    out.append(("eof", "", -1))
    return out


# --------------------------------------------------------------------- parser

class _Parser:
    def __init__(self, text):
        self.t = tokenize(text)
        self.i = 0

    def peek(self, k=0):
        return self.t[self.i + k]

    def take(self, value=None, kind=None):
        tok = self.t[self.i]
        if (value is not None and tok[1] != value) or (kind is not None and tok[0] != kind):
            want = value if value is not None else kind
            raise DslError(f"line {tok[2]}: expected {want!r}, found {tok[1]!r}")
        self.i += 1
        return tok

    def accept(self, value):
        if self.t[self.i][1] == value:
            self.i += 1
            return True
        return False

    # grammar := (axiom | terminal | rule)*
    def grammar(self):
        g = {"axioms": [], "terminals": {}, "rules": {}, "order": []}
        while self.peek()[0] != "eof":
            tok = self.peek()
            if tok[1] == "axiom":
                self.take()
                shape = self.take(kind="name")[1]
                if shape not in SHAPES:
                    raise DslError(f"line {tok[2]}: unknown axiom shape {shape!r}")
                name = self.take(kind="name")[1]
                self.take(";")
                g["axioms"].append((shape, name))
            elif tok[1] == "terminal":
                self.take()
                names = []
                while self.peek()[0] == "name":
                    names.append(self.take()[1])
                self.take("(")
                args = [self.number()]
                while self.accept(","):
                    args.append(self.number())
                self.take(")")
                self.take(";")
                for n in names:
                    g["terminals"][n] = tuple(args)
            else:
                name = self.take(kind="name")[1]
                self.take("=")
                chain = self.chain()
                self.take(";")
                if name in g["rules"]:
                    raise DslError(f"line {tok[2]}: rule {name!r} defined twice")
                g["rules"][name] = chain
                g["order"].append(name)
        return g

    def number(self):
        neg = self.accept("-")
        v = float(self.take(kind="num")[1])
        return -v if neg else v

    # chain := (operator)* (name | block-ending operator)
    def chain(self):
        ops = []
        while True:
            tok = self.peek()
            if tok[0] != "name":
                raise DslError(f"line {tok[2]}: expected an operator or a symbol, found {tok[1]!r}")
            if self.peek(1)[1] != "(":
                self.take()
                ops.append(("symbol", tok[1], tok[2]))
                return ops
            name = self.take()[1]
            args = self.args()
            if name == "Discard":
                ops.append(("op", name, args, None, tok[2]))
                return ops
            if self.peek()[1] == "{" or name in BRANCHING:
                ops.append(("op", name, args, self.block(name), tok[2]))
                return ops
            ops.append(("op", name, args, None, tok[2]))

    def block(self, name):
        self.take("{")
        succ = []
        while True:
            factor = None
            if name in ("SubDiv", "RandomRule"):  # size factor / selection weight
                factor = self.arg()
                self.take(":")
            succ.append((factor, self.chain()))
            if self.accept("|"):
                continue
            self.take("}")
            return succ

    def args(self):
        self.take("(")
        out = []
        if self.accept(")"):
            return out
        out.append(self.arg())
        while self.accept(","):
            out.append(self.arg())
        self.take(")")
        return out

    # arg := number | axis | mode | function(...) | (tuple)
    def arg(self):
        tok = self.peek()
        if tok[1] == "-" or tok[0] == "num":
            return ("num", self.number())
        if tok[1] == "(":
            self.take("(")
            vals = [self.arg()]
            while self.accept(","):
                vals.append(self.arg())
            self.take(")")
            return ("tuple", vals)
        name = self.take(kind="name")[1]
        if name in AXES:
            return ("axis", AXES[name])
        if name in MODES:
            return ("mode", MODES[name])
        if name == "Exp":
            self.take("(")
            e = self.expr()
            self.take(")")
            return ("exp", e)
        args = self.args()
        return ("fn", name, args)

    # infix expression: or > and > comparison > additive > multiplicative > unary
    def expr(self):
        return self._binary(0)

    _LEVELS = [("||",), ("&&",), ("==", "!=", "<", ">", "<=", ">="), ("+", "-"), ("*", "/")]

    def _binary(self, level):
        if level == len(self._LEVELS):
            return self._unary()
        left = self._binary(level + 1)
        while self.peek()[1] in self._LEVELS[level]:
            op = self.take()[1]
            right = self._binary(level + 1)
            left = ("bin", op, left, right)
        return left

    def _unary(self):
        tok = self.peek()
        if tok[1] == "-" and self.peek(1)[0] == "num":
            return ("num", self.number())
        if tok[1] == "(":
            self.take("(")
            e = self.expr()
            self.take(")")
            return e
        if tok[0] == "num":
            return ("num", self.number())
        return self.arg()


def parse(text):
    """Syntax tree of a .pga grammar: {"axioms", "terminals", "rules", "order"}."""
    return _Parser(text).grammar()


# ------------------------------------------------------------------- lowering

_OPCODE = {"+": G.OPT_ADD, "-": G.OPT_SUB, "/": G.OPT_DIV, "*": G.OPT_MULTI, "==": G.OPT_EQ, "!=": G.OPT_NEQ,
           "<": G.OPT_LT, ">": G.OPT_GT, "<=": G.OPT_LEQ, ">=": G.OPT_GEQ, "&&": G.OPT_AND, "||": G.OPT_OR}


def _attr_index(fn, args):
    """Shape attribute index of a Shape* function (Parameters.cuh:123-199)."""
    a = args[0][1] if args else 0
    if fn == "ShapeSize":
        return 12 + a
    if fn == "ShapeNormal":
        return a * 4 + 2
    if fn == "ShapePos":
        return (a + 1) * 4 - 1
    if fn == "ShapeSeed":
        return 15
    if fn == "ShapeCustomAttribute":
        return 16
    raise DslError(f"{fn}() is not a shape attribute")


def _postfix(e, out):
    kind = e[0]
    if kind == "num":
        out.append(("s", e[1]))
    elif kind == "axis" or kind == "mode":
        out.append(("s", float(e[1])))
    elif kind == "fn" and e[1].startswith("Shape"):
        out.append(("a", _attr_index(e[1], e[2])))
    elif kind == "bin":
        _postfix(e[2], out)
        _postfix(e[3], out)
        out.append(("op", _OPCODE[e[1]]))
    else:
        raise DslError(f"unsupported expression operand {e!r}")
    return out


def _param(arg):
    kind = arg[0]
    if kind in ("num",):
        return G.scalar(arg[1])
    if kind in ("axis", "mode"):
        return G.scalar(float(arg[1]))
    if kind == "exp":
        e = arg[1]
        if e[0] == "num":
            return G.scalar(e[1])
        return G.exp(*_postfix(e, []))
    if kind == "fn":
        if arg[1].startswith("Shape"):
            return G.shape_attr(_attr_index(arg[1], arg[2]))
        if arg[1] == "Rand":
            return G.rand(arg[2][0][1], arg[2][1][1])
    raise DslError(f"unsupported parameter {arg!r}")


class _Lowering:
    def __init__(self, g):
        self.g = g
        self.entries = []
        self.memo = {}  # (rule, shape) -> entry index

    def new(self):
        self.entries.append(None)
        return len(self.entries) - 1

    def rule(self, name, shape, line):
        if name in self.g["terminals"]:
            fn, *rest = self.g["terminals"][name]
            if int(fn) not in (0, 1):
                raise DslError(f"terminal {name!r}: generation function {int(fn)}; only 0 (triangle mesh) and 1 "
                               "(instanced) are supported")
            key = ("terminal", name, shape)
            if key not in self.memo:
                i = self.new()
                self.memo[key] = i
                if int(fn) == 1:
                    gen = G.BOX_GENERATE if shape == G.SHAPE_BOX else G.QUAD_GENERATE
                else:
                    gen = G.BOX_GENERATE_MESH if shape == G.SHAPE_BOX else G.QUAD_GENERATE_MESH
                self.entries[i] = G.Entry(gen, [G.scalar(rest[0] if rest else 0.0)], [])
            return self.memo[key]
        if name not in self.g["rules"]:
            raise DslError(f"line {line}: unknown symbol {name!r}")
        key = (name, shape)
        if key not in self.memo:
            i = self.new()
            self.memo[key] = i  # before lowering the body: recursion refers back to it
            self.chain_into(i, self.g["rules"][name], shape, name)
        return self.memo[key]

    def chain(self, ops, shape, rule):
        """Entry index of a chain applied to `shape` (a fresh entry per inline chain)."""
        if len(ops) == 1 and ops[0][0] == "symbol":
            return self.rule(ops[0][1], shape, ops[0][2])
        i = self.new()
        self.chain_into(i, ops, shape, rule)
        return i

    def chain_into(self, i, ops, shape, rule):
        head = ops[0]
        if head[0] == "symbol":
            # an alias rule (A = B;) takes over B's entry definition
            j = self.rule(head[1], shape, head[2])
            self.entries[i] = self.entries[j]
            return
        _, name, args, block, line = head
        rest = ops[1:]
        where = f"rule {rule!r} (line {line})"
        if name not in SUPPORTED:
            raise DslError(f"{where}: operator {name} is not supported by the GB300 engine")
        box = shape == G.SHAPE_BOX
        if name == "Discard":
            self.entries[i] = G.Entry(G.BOX_DISCARD if box else G.QUAD_DISCARD, [], [])
        elif name == "SubDiv":
            params = [_param(args[0])] + [_param(f) for f, _ in block]
            succ = [(self.chain(c, shape, rule), 0) for _, c in block]
            self.entries[i] = G.Entry(G.BOX_SUBDIVIDE if box else G.QUAD_SUBDIVIDE, params, succ)
        elif name == "Repeat":
            if not rest:
                raise DslError(f"{where}: Repeat needs a successor")
            params = [_param(a) for a in args[:3]]
            if len(params) == 2:
                params.append(G.scalar(float(G.ANCHOR_TO_START)))
            self.entries[i] = G.Entry(G.BOX_REPEAT if box else G.QUAD_REPEAT, params,
                                      [(self.chain(rest, shape, rule), 0)])
        elif name == "CompSplit":
            if not box:
                raise DslError(f"{where}: CompSplit needs a Box")
            succ = [(self.chain(c, G.SHAPE_QUAD, rule), 0) for _, c in block]
            if len(succ) != 3:
                raise DslError(f"{where}: CompSplit takes three successors (top | bottom | sides)")
            self.entries[i] = G.Entry(G.BOX_COMPONENT_SPLIT, [], succ)
        elif name == "Extrude":
            if box:
                raise DslError(f"{where}: Extrude needs a Quad")
            if not rest:
                raise DslError(f"{where}: Extrude needs a successor")
            extent = _param(args[-1])
            axis = _param(args[0]) if len(args) > 1 else G.scalar(0.0)  # the axis slot is unused
            self.entries[i] = G.Entry(G.QUAD_EXTRUDE, [axis, extent], [(self.chain(rest, G.SHAPE_BOX, rule), 0)])
        elif name in ("Translate", "Scale", "Rotate", "SwapSize"):
            if not rest:
                raise DslError(f"{where}: {name} needs a successor")
            if len(args) < 3:
                raise DslError(f"{where}: {name} takes three parameters (x, y, z)")
            if name == "Translate":
                op = G.BOX_TRANSLATE if box else G.QUAD_TRANSLATE
            elif name == "Scale":
                op = G.BOX_SCALE if box else G.QUAD_SCALE
            elif name == "SwapSize":
                op = G.BOX_SWAP_SIZE if box else G.QUAD_SWAP_SIZE
            else:
                op = G.BOX_ROTATE if box else G.QUAD_ROTATE
            self.entries[i] = G.Entry(op, [_param(a) for a in args[:3]], [(self.chain(rest, shape, rule), 0)])
        elif name == "RandomRule":
            if not args:
                raise DslError(f"{where}: RandomRule takes the chance as its parameter")
            if not block:
                raise DslError(f"{where}: RandomRule needs weighted successors (weight: successor | ...)")
            params = [_param(args[0])] + [_param(f) for f, _ in block]
            succ = [(self.chain(c, shape, rule), 0) for _, c in block]
            self.entries[i] = G.Entry(G.BOX_RANDOM_RULE if box else G.QUAD_RANDOM_RULE, params, succ)
        elif name == "Replicate":
            if not block:
                raise DslError(f"{where}: Replicate needs successors ({{ a | b | ... }})")
            succ = [(self.chain(c, shape, rule), 0) for _, c in block]
            self.entries[i] = G.Entry(G.BOX_REPLICATE if box else G.QUAD_REPLICATE, [], succ)
        elif name == "If":
            succ = [(self.chain(c, shape, rule), 0) for _, c in block]
            if len(succ) != 2 or not args:
                raise DslError(f"{where}: If takes a condition and two successors (true | false)")
            self.entries[i] = G.Entry(G.BOX_IF if box else G.QUAD_IF, [_param(args[0])], succ)
        elif name == "IfSizeLess":
            succ = [(self.chain(c, shape, rule), 0) for _, c in block]
            if len(succ) != 2:
                raise DslError(f"{where}: IfSizeLess takes two successors (true | false)")
            self.entries[i] = G.Entry(G.BOX_IF_SIZE_LESS if box else G.QUAD_IF_SIZE_LESS,
                                      [_param(args[0]), _param(args[1])], succ)


def lower(g):
    """Dispatch table (ENTRY_DT array on grammar.DEFAULT_PROCS) of a parsed
    grammar, and the axioms' (shape, entry) pairs."""
    if not g["axioms"]:
        raise DslError("the grammar has no axiom")
    L = _Lowering(g)
    roots = [(SHAPES[s], L.rule(name, SHAPES[s], 0)) for s, name in g["axioms"]]
    if any(e is None for e in L.entries):
        raise DslError("a rule is defined only through itself")
    return G.DispatchTable(L.entries).to_array(), roots


def load(text, n_axioms=1):
    """Parses and lowers `text`; returns a scenes-style batch with `n_axioms`
    unit axioms of the first axiom declaration (sizes, positions, seeds to be
    set by the caller)."""
    entries, roots = lower(parse(text))
    shape, entry = roots[0]
    ax = G.make_axioms(n_axioms)
    ax["shape"] = shape
    ax["entry"] = entry
    ax["size"] = 1.0
    return {"entries": entries, "axioms": ax, "blocks": None, "block_stride": 0, "name": "pga"}
