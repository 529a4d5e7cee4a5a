"""A front end for Simit element functions: `.sim` source -> the CUDA C++
element function of the run-time compiled assembly (sg_jit_assembly_create).

The reference compiles a whole Simit program (src/frontend/parser.cpp,
src/frontend/ir_emitter.cpp), inlines the function of a `map f to E reduce +`
into the element loop (src/inline.cpp:690-888) and turns its writes into
`+=` on the matrix slots (src/lower/lower_maps.cpp:54-128).  This module
covers the part of that pipeline an element function of such a map needs:

* a parser for the language's declarations, functions, statements and
  expressions: element and extern declarations, `func` with scalar,
  element, endpoint-tuple and tensor arguments (tensor, vector and matrix
  types, nested block types), `var` / `const`, assignment, indexed and
  multiple assignment, `for`, `while`, `if` / `elif` / `else`, `apply`,
  tensor literals, transpose, slices, calls, field access,
  `map ... to ... reduce +`;
* a generator that turns one element function of a map into the element
  function the run-time compiled assembly takes.  The function body runs
  as written on local arrays.  For a matrix result, every write
  `K(v(a), v(b)) = value` becomes a term of block (i, j) of
  `element_block(e, i, j, ep, f, blk)` when (a, b) == (i, j); for a vector
  result, every write `f(v(a)) = value` a term of endpoint i of
  `element_vector(e, i, ep, f, vec)` when a == i.  Terms keep statement
  order -- one `+=` each, as the lowered map does.  A write of one
  component, `K(v(a), v(b))(r, c) = x` or `f(v(a))(r) = x`, adds x there
  only; a scalar written to a block or a vector fills it.  Dense tensor products are emitted as the lowered loops compute
  them (each entry summed from zero over the inner index in ascending
  order), scalar-tensor and element-wise operations entry by entry, so with
  contraction off (the run-time compiler's exact mode) the values follow
  the program's operation order.  det and inv of 3x3 matrices follow the
  reference runtime's cofactor formulas (src/runtime.cpp:90-94, 147-173).

Element fields (`e.B`, `e.W`) and endpoint fields (`v(i).x`, `v(i).c`)
become the assembly's field arrays in first-use order (`fields` of the
result); the map's scalar arguments (`compute_stiffness(h)`) are bound to
constants.  A map over a vertex set (`func f(p : Point) -> K(p, p) = ...`)
compiles with one endpoint per element: assemble it over a mesh whose
elements are the vertices themselves.

The generated function recomputes the element's work for each block it is
asked for; it is the general path for programs without a hand-written
kernel, not a replacement for the precompiled element kernels.
"""
import re

import numpy as np

KEYWORDS = {"func", "proc", "end", "for", "in", "if", "elif", "else", "var", "const", "and",
            "or", "xor", "not", "element", "extern", "export", "set", "tensor", "vector",
            "matrix", "float", "double", "int", "bool", "string", "complex", "map", "to",
            "reduce", "while", "inout", "true", "false", "print", "println", "return", "apply",
            "grid", "ivar", "do"}


class SimError(Exception):
    pass


MAX_FIELDS = 8      # field arrays the run-time compiled assembly takes


# ---------------------------------------------------------------------------
# lexer
# ---------------------------------------------------------------------------
_TOKEN = re.compile(r"""
    (?P<ws>\s+) | (?P<bcomment>(?s:%\{.*?%\})) | (?P<comment>%[^\n]*) |
    (?P<num>(\d+\.\d*|\.\d+|\d+)([eE][+-]?\d+)?) |
    (?P<str>"[^"\n]*") |
    (?P<id>[A-Za-z_][A-Za-z0-9_]*) |
    (?P<op>==|!=|<=|>=|->|\.\*|\./|[-+*/'=<>(),;:.\[\]{}\\^])
""", re.X)


def tokenize(src):
    """[(kind, text, line)] ending with ("eof", "", line)."""
    out, pos, line = [], 0, 1
    while pos < len(src):
        m = _TOKEN.match(src, pos)
        if not m:
            raise SimError("line %d: unexpected %r" % (line, src[pos]))
        kind = m.lastgroup
        text = m.group(kind)
        if kind == "id" and text in KEYWORDS:
            kind = "kw"
        if kind not in ("ws", "comment", "bcomment"):
            out.append((kind, text, line))
        line += text.count("\n")
        pos = m.end()
    out.append(("eof", "", line))
    return out


# ---------------------------------------------------------------------------
# parser (nodes are tuples whose first entry names the kind)
# ---------------------------------------------------------------------------
_SCALARS = ("float", "double", "int", "bool", "string", "complex")


class Parser:
    def __init__(self, src):
        self.t = tokenize(src)
        self.i = 0

    def peek(self, k=0):
        return self.t[min(self.i + k, len(self.t) - 1)]

    def take(self, text=None, kind=None):
        tk = self.t[self.i]
        if (text is not None and tk[1] != text) or (kind is not None and tk[0] != kind):
            raise SimError("line %d: expected %s, found %r" % (tk[2], text or kind, tk[1]))
        self.i += 1
        return tk

    def at(self, text):
        return self.t[self.i][1] == text and self.t[self.i][0] != "str"

    def accept(self, text):
        if self.at(text):
            self.i += 1
            return True
        return False

    # program ----------------------------------------------------------------
    def program(self):
        prog = {"elements": {}, "externs": {}, "funcs": {}, "consts": {}, "extern_funcs": {}}
        while self.peek()[0] != "eof":
            if self.accept("element"):
                name = self.take(kind="id")[1]
                fields = {}
                while not self.at("end"):
                    fname = self.take()[1]          # keywords are valid field names
                    self.take(":")
                    fields[fname] = self.type_()
                    self.take(";")
                self.take("end")
                prog["elements"][name] = fields
            elif self.accept("extern"):
                if self.at("func") or self.at("proc"):
                    f = self.header()
                    self.take(";")
                    prog["extern_funcs"][f["name"]] = f
                    continue
                name = self.take(kind="id")[1]
                self.take(":")
                prog["externs"][name] = self.type_()
                self.take(";")
            elif self.accept("const"):
                name = self.take(kind="id")[1]
                ty = self.type_() if self.accept(":") else None
                self.take("=")
                prog["consts"][name] = (ty, self.expr())
                self.take(";")
            else:
                self.accept("export")
                f = self.header()
                f["body"] = self.stmts(("end",))
                self.take("end")
                prog["funcs"][f["name"]] = f
        return prog

    def header(self):
        if not self.accept("proc"):
            self.take("func")
        name = self.take(kind="id")[1]
        if self.accept("<"):
            while not self.accept(">"):
                self.take()
        args = []
        if self.accept("("):
            while not self.at(")"):
                inout = self.accept("inout")
                an = self.take(kind="id")[1]
                self.take(":")
                args.append((an, self.type_(), inout))
                if not self.accept(","):
                    break
            self.take(")")
        results = []
        if self.accept("->"):
            paren = self.accept("(")
            while True:
                rn = self.take(kind="id")[1]
                self.take(":")
                results.append((rn, self.type_()))
                if not paren or not self.accept(","):
                    break
            if paren:
                self.take(")")
        return {"name": name, "args": args, "results": results}

    def type_(self):
        tk = self.peek()
        if tk[1] in _SCALARS:
            self.i += 1
            return ("scalar", "float" if tk[1] == "double" else tk[1])
        if tk[1] in ("tensor", "vector", "matrix"):
            self.i += 1
            dims = []
            if self.accept("["):
                while True:
                    d = self.take()
                    dims.append(int(d[1]) if d[0] == "num" else d[1])
                    if not self.accept(","):
                        break
                self.take("]")
            self.take("(")
            inner = self.type_()
            self.take(")")
            col = not self.accept("'")
            if not dims:
                return inner
            return ("tensor", tuple(dims), inner, col)
        if tk[1] in ("set", "grid"):
            self.i += 1
            if tk[1] == "grid":
                self.take("[")
                self.take(kind="num")
                self.take("]")
            self.take("{")
            el = self.take(kind="id")[1]
            self.take("}")
            return ("set", el, self.endpoint_list())
        if tk[1] == "(":
            self.take("(")
            if self.peek(1)[1] == "*":
                el = self.take(kind="id")[1]
                self.take("*")
                k = int(self.take(kind="num")[1])
                self.take(")")
                return ("tuple", ((None, el),) * k)
            members = []
            while not self.at(")"):
                if self.peek(1)[1] == ":":
                    mn = self.take(kind="id")[1]
                    self.take(":")
                else:
                    mn = None
                members.append((mn, self.take(kind="id")[1]))
                if not self.accept(","):
                    break
            self.take(")")
            return ("tuple", tuple(members))
        if tk[1] == "subsetof":     # `subsetof points{2}`: endpoints from a set
            self.i += 1
            setname = self.take(kind="id")[1]
            self.take("{")
            k = int(self.take(kind="num")[1])
            self.take("}")
            return ("tuple", (("@set", setname),) * k)
        if tk[0] == "id":
            self.i += 1
            if self.accept("["):    # `Spring[points, points]{}`: a lattice set
                while not self.accept("]"):
                    self.take()
            if self.at("{"):        # `Point{}` / `Link{}(points)`: a set
                self.take("{")
                self.take("}")
                return ("set", tk[1], self.endpoint_list())
            return ("element", tk[1])
        raise SimError("line %d: expected a type, found %r" % (tk[2], tk[1]))

    def endpoint_list(self):
        eps = []
        if self.accept("("):
            while not self.at(")"):
                ep = self.take(kind="id")[1]
                k = 1
                if self.accept("*"):            # set{Edge}(V*2)
                    k = int(self.take(kind="num")[1])
                eps.extend([ep] * k)
                if not self.accept(","):
                    break
            self.take(")")
        return tuple(eps)

    # statements -------------------------------------------------------------
    def stmts(self, stops):
        out = []
        while self.peek()[1] not in stops or self.peek()[0] == "str":
            if self.peek()[0] == "eof":
                raise SimError("unexpected end of the program")
            out.append(self.stmt())
        return out

    def stmt(self):
        tk = self.peek()
        line = tk[2]
        if tk[1] in ("var", "const") and tk[0] == "kw":
            self.i += 1
            name = self.take(kind="id")[1]
            ty = self.type_() if self.accept(":") else None
            init = self.expr() if self.accept("=") else None
            self.take(";")
            return ("var", name, ty, init, line)
        if tk[1] == "ivar":
            self.i += 1
            while not self.accept(";"):
                self.take()
            return ("nop", line)
        if tk[1] == "for":
            self.take("for")
            var = self.take(kind="id")[1]
            self.take("in")
            lo = self.expr()
            hi = None
            if self.accept(":"):
                hi = self.expr()
            body = self.stmts(("end",))
            self.take("end")
            if hi is None:
                return ("forset", var, lo, body, line)
            return ("for", var, lo, hi, body, line)
        if tk[1] == "do":
            self.take("do")
            body = self.stmts(("end",))
            self.take("end")
            self.take("while")
            cond = self.expr()
            self.accept(";")
            return ("dowhile", cond, body, line)
        if tk[1] == "while":
            self.take("while")
            cond = self.expr()
            body = self.stmts(("end",))
            self.take("end")
            return ("while", cond, body, line)
        if tk[1] == "if":
            self.take("if")
            arms = [(self.expr(), self.stmts(("elif", "else", "end")))]
            els = []
            while True:
                if self.accept("elif"):
                    c = self.expr()
                    arms.append((c, self.stmts(("elif", "else", "end"))))
                    continue
                if self.accept("else"):
                    els = self.stmts(("end",))
                self.take("end")
                break
            return ("if", arms, els, line)
        if tk[1] in ("print", "println"):
            self.i += 1
            args = [self.expr()]
            while self.accept(","):
                args.append(self.expr())
            self.take(";")
            return ("print", args, line)
        if tk[1] == "return":
            self.take("return")
            self.take(";")
            return ("return", line)
        if tk[1] == "apply":
            self.take("apply")
            fn = self.take(kind="id")[1]
            args = self.call_args() if self.at("(") else []
            self.take("to")
            target = self.take(kind="id")[1]
            self.take(";")
            return ("apply", fn, args, target, line)
        lhs = [self.expr()]
        while self.accept(","):
            lhs.append(self.expr())
        if self.accept("="):
            rhs = self.expr()
            self.take(";")
            if len(lhs) > 1:
                return ("massign", lhs, rhs, line)
            return ("assign", lhs[0], rhs, line)
        self.take(";")
        if len(lhs) > 1:
            raise SimError("line %d: a list of expressions is not a statement" % line)
        return ("expr", lhs[0], line)

    # expressions ------------------------------------------------------------
    def call_args(self):
        self.take("(")
        args = []
        while not self.at(")"):
            if self.at(":") and self.peek(1)[1] in (",", ")"):
                self.take(":")
                args.append(("slice",))
            else:
                args.append(self.expr())
            if not self.accept(","):
                break
        self.take(")")
        return args

    def expr(self):
        if self.accept("map"):
            fn = self.take(kind="id")[1]
            args = self.call_args() if self.at("(") else []
            self.take("to")
            target = self.take(kind="id")[1]
            if self.peek()[1] == "through":     # stencil map over a lattice
                self.take()
                target = (target, self.take(kind="id")[1])
            if self.peek()[1] == "with":        # the endpoint set of a lattice map
                self.take()
                self.take(kind="id")
            red = None
            if self.accept("reduce"):
                red = self.take()[1]
            return ("map", fn, args, target, red)
        return self.or_()

    def or_(self):
        e = self.xor_()
        while self.accept("or"):
            e = ("bin", "or", e, self.xor_())
        return e

    def xor_(self):
        e = self.and_()
        while self.accept("xor"):
            e = ("bin", "xor", e, self.and_())
        return e

    def and_(self):
        e = self.not_()
        while self.accept("and"):
            e = ("bin", "and", e, self.not_())
        return e

    def not_(self):
        if self.accept("not"):
            return ("un", "not", self.not_())
        return self.cmp()

    def cmp(self):
        e = self.add()
        while self.peek()[1] in ("==", "!=", "<", ">", "<=", ">="):
            op = self.take()[1]
            e = ("bin", op, e, self.add())
        return e

    def add(self):
        e = self.mul()
        while self.peek()[1] in ("+", "-") and self.peek()[0] == "op":
            op = self.take()[1]
            e = ("bin", op, e, self.mul())
        return e

    def mul(self):
        e = self.unary()
        while self.peek()[1] in ("*", "/", ".*", "./", "\\") and self.peek()[0] == "op":
            op = self.take()[1]
            e = ("bin", op, e, self.unary())
        return e

    def unary(self):
        if self.accept("-"):
            return ("un", "-", self.unary())
        if self.accept("+"):
            if self.peek()[0] == "id" and self.peek(1)[0] == "id":
                ivar = self.take()[1]           # `+i a{i} * b{i}`: a sum over i
                return ("isum", ivar, self.unary_chain())
            return self.unary()
        e = self.postfix()
        if self.accept("^"):
            return ("bin", "^", e, self.unary())
        return e

    def unary_chain(self):
        e = self.unary()
        while self.peek()[1] in ("*", "/", ".*", "./") and self.peek()[0] == "op":
            op = self.take()[1]
            e = ("bin", op, e, self.unary())
        return e

    def postfix(self):
        e = self.primary()
        while True:
            if self.at("'"):
                self.take("'")
                e = ("tr", e)
            elif self.at("("):
                e = ("call", e, self.call_args())
            elif self.at(".") and self.peek(1)[0] in ("id", "kw"):
                self.take(".")
                e = ("field", e, self.take()[1])
            elif self.at("{") and e[0] in ("name", "field"):   # index notation c{i}
                self.take("{")
                ivars = []
                while not self.accept("}"):
                    if not self.accept(","):
                        ivars.append(self.take(kind="id")[1])
                e = ("ivar", e, ivars)
            elif self.at("["):                  # lattice access l[0,0; 0,1]
                self.take("[")
                offs = []
                while not self.accept("]"):
                    if self.accept(",") or self.accept(";"):
                        continue
                    offs.append(self.add())
                e = ("lattice", e, offs)
            else:
                return e

    def generic_args(self):
        """Skips `<a, b>` when a call's argument list follows it."""
        j = self.i + 1
        while j < len(self.t) and (self.t[j][0] in ("id", "num") or self.t[j][1] in (",", "-")):
            j += 1
        if j < len(self.t) and self.t[j][1] == ">" and j + 1 < len(self.t) and \
                self.t[j + 1][1] == "(":
            self.i = j + 1
            return True
        return False

    def primary(self):
        tk = self.peek()
        if tk[0] == "num":
            self.i += 1
            isf = any(ch in tk[1] for ch in ".eE")
            return ("num", float(tk[1]) if isf else int(tk[1]), isf)
        if tk[1] in ("true", "false") and tk[0] == "kw":
            self.i += 1
            return ("bool", tk[1] == "true")
        if tk[0] == "id":
            self.i += 1
            if self.at("<") and self.generic_args():
                pass                            # foo<5, 6>(a): explicit generic arguments
            return ("name", tk[1])
        if self.at("<"):                        # complex literal <re, im>
            self.take("<")
            re_ = self.add()
            self.take(",")
            im = self.add()
            self.take(">")
            return ("complex", re_, im)
        if tk[0] == "str":
            self.i += 1
            return ("str", tk[1][1:-1])
        if self.accept("("):
            e = self.expr()
            self.take(")")
            return e
        if self.accept("["):
            rows, row = [], []
            while True:
                if self.at("["):          # nested literal: [[1, 2], [3, 4]]
                    row.append(self.primary())
                else:
                    row.append(self.expr())
                if self.accept(","):
                    continue
                if self.accept(";"):
                    rows.append(row)
                    row = []
                    continue
                if self.accept("]"):
                    rows.append(row)
                    break
                # space-separated entries: [1.0 0.0; 0.0 1.0]
            return ("lit", rows)
        raise SimError("line %d: unexpected %r" % (tk[2], tk[1]))


def parse(src):
    """The program as {"elements", "externs", "funcs", "consts",
    "extern_funcs"} of nodes."""
    return Parser(src).program()


# ---------------------------------------------------------------------------
# code generation
# ---------------------------------------------------------------------------
class _Val:
    """A generated value.  kind: 'scalar' (C expression of type real), 'int',
    'bool' (C expressions), 'tensor' (C array `real name[size]`, row-major,
    shape: (rows, cols) for matrices and vectors -- a column vector is
    (n, 1) -- or the dimensions of a higher-order tensor), 'vertex' (C
    expression of the local endpoint index; elem: the element type),
    'element' (the map's element), 'tuple' (the endpoints)."""

    def __init__(self, kind, code=None, shape=None, elem=None):
        self.kind, self.code, self.shape, self.elem = kind, code, shape, elem


def _size(shape):
    n = 1
    for d in shape:
        n *= d
    return n


def _lit(x):
    return "real(%r)" % float(x)


_MATH1 = {"sqrt": "sqrt", "log": "log", "exp": "exp", "sin": "sin", "cos": "cos", "tan": "tan",
          "asin": "asin", "acos": "acos", "atan": "atan", "abs": "fabs"}

# det and inv of a 3x3 matrix: cofactors, one reciprocal, products (the
# reference runtime's det3 / inv3, src/runtime.cpp:90-94 and 147-173)
_INTRINSICS = {
    "det3": r"""
__device__ inline real simi_det3(const real *a) {
  return a[0] * (a[4] * a[8] - a[5] * a[7]) - a[1] * (a[3] * a[8] - a[5] * a[6]) +
         a[2] * (a[3] * a[7] - a[4] * a[6]);
}
""",
    "inv3": r"""
__device__ inline void simi_inv3(const real *a, real *o) {
  const real c00 = a[4] * a[8] - a[5] * a[7], c01 = -a[3] * a[8] + a[5] * a[6];
  const real c02 = a[3] * a[7] - a[4] * a[6], c10 = -a[1] * a[8] + a[2] * a[7];
  const real c11 = a[0] * a[8] - a[2] * a[6], c12 = -a[0] * a[7] + a[1] * a[6];
  const real c20 = a[1] * a[5] - a[2] * a[4], c21 = -a[0] * a[5] + a[2] * a[3];
  const real c22 = a[0] * a[4] - a[1] * a[3];
  const real r = real(1.0) / (a[0] * c00 + a[1] * c01 + a[2] * c02);
  o[0] = c00 * r; o[1] = c10 * r; o[2] = c20 * r;
  o[3] = c01 * r; o[4] = c11 * r; o[5] = c21 * r;
  o[6] = c02 * r; o[7] = c12 * r; o[8] = c22 * r;
}
""",
}


def _shape_of_type(ty):
    """Local shape of a tensor type (() for scalars); nested block types
    (tensor[3](tensor[3](float))) flatten to their combined dimensions."""
    if ty[0] == "scalar":
        return ()
    if ty[0] != "tensor":
        raise SimError("type %r has no local shape" % (ty,))
    dims, inner, col = ty[1], ty[2], ty[3]
    if any(not isinstance(d, int) for d in dims):
        raise SimError("a system tensor cannot be a local value")
    ishape = _shape_of_type(inner)
    if len(dims) == 1 and not ishape:
        return (dims[0], 1) if col else (1, dims[0])
    if ishape:
        ishape = tuple(d for d in ishape if d != 1) or (1,)
        return tuple(dims) + ishape
    return tuple(dims)


class _Gen:
    def __init__(self, prog, consts, state=None):
        self.prog = prog
        self.consts = dict(consts)
        self.lines = []
        self.ind = 1
        self.ntmp = 0
        self.results = {}
        self.target = None
        self.vertex_map = False
        self.vector = False
        self.nest = None
        self.cwords = 1
        # shared between an element function and its helpers
        self.st = state if state is not None else {
            "fields": [], "field_index": {}, "funcs_out": [], "funcs_done": {},
            "intrinsics": []}

    # helpers ----------------------------------------------------------------
    def emit(self, s):
        self.lines.append("  " * self.ind + s)

    def tmp(self, prefix="t"):
        self.ntmp += 1
        return "%s%d_" % (prefix, self.ntmp)

    def new_tensor(self, shape, prefix="t"):
        name = self.tmp(prefix)
        self.emit("real %s[%d];" % (name, _size(shape)))
        return name

    def intrinsic(self, key):
        if key not in self.st["intrinsics"]:
            self.st["intrinsics"].append(key)

    def as_scalar(self, v, what="value"):
        if v.kind in ("scalar", "int", "bool"):
            return v.code
        if v.kind == "tensor" and _size(v.shape) == 1:
            return "%s[0]" % v.code
        raise SimError("%s: a scalar is needed" % what)

    def elementwise(self, shape, fn):
        out = self.new_tensor(shape)
        self.emit("for (int q_ = 0; q_ < %d; ++q_) %s[q_] = %s;" % (_size(shape), out, fn("q_")))
        return _Val("tensor", out, shape)

    def is_tensor(self, v):
        return v.kind == "tensor" and _size(v.shape) != 1

    # fields -----------------------------------------------------------------
    def field_info(self, kind, elem, name):
        fields = self.prog["elements"].get(elem)
        if fields is None or name not in fields:
            raise SimError("%s has no field %r" % (elem, name))
        key = (kind, name)
        st = self.st
        if key not in st["field_index"]:
            fty = fields[name]
            if fty[0] == "scalar":
                shape, dt = (), fty[1]
            else:
                shape = _shape_of_type(fty)
                inner = fty[2]
                while inner[0] == "tensor":
                    inner = inner[2]
                dt = inner[1]
            st["field_index"][key] = len(st["fields"])
            st["fields"].append((kind, name, shape, dt))
        k = st["field_index"][key]
        _, _, shape, dt = st["fields"][k]
        ctype = {"int": "int", "bool": "bool"}.get(dt, "real")
        return "reinterpret_cast<const %s *>(f[%d])" % (ctype, k), shape, dt

    def arg_field(self, name, shape, dt):
        """A map argument that is a system vector (`map f(y) to V`, y a
        tensor[V](...)): passed like a vertex field, as ("arg", name)."""
        key = ("arg", name)
        st = self.st
        if key not in st["field_index"]:
            st["field_index"][key] = len(st["fields"])
            st["fields"].append(("arg", name, shape, dt))
        k = st["field_index"][key]
        ctype = {"int": "int", "bool": "bool"}.get(dt, "real")
        return "reinterpret_cast<const %s *>(f[%d])" % (ctype, k)

    def sysvec_read(self, v, args, env):
        """y(p) of a system-vector argument: the block of vertex p (the
        map's element in a map over the vertices, else an endpoint)."""
        if len(args) != 1:
            raise SimError("a system vector is indexed by one vertex")
        p = self.expr(args[0], env)
        if p.kind == "element" and self.vertex_map:
            idx = "e"
        elif p.kind == "vertex":
            idx = "ep[%s]" % p.code
        else:
            raise SimError("a system vector is indexed by a vertex")
        ptr = self.arg_field(v.code, v.shape, v.elem)
        if v.shape == ():
            return _Val({"int": "int", "bool": "bool"}.get(v.elem, "scalar"),
                        "%s[%s]" % (ptr, idx))
        out = self.new_tensor(v.shape)
        sz = _size(v.shape)
        self.emit("for (int q_ = 0; q_ < %d; ++q_) %s[q_] = %s[(long long)%s * %d + q_];"
                  % (sz, out, ptr, idx, sz))
        return _Val("tensor", out, v.shape)

    def field_base(self, e, env):
        base = self.expr(e[1], env)
        if base.kind == "element":
            ptr, shape, dt = self.field_info("element", base.elem, e[2])
            return ptr, shape, dt, "e"
        if base.kind == "vertex":
            ptr, shape, dt = self.field_info("vertex", base.elem, e[2])
            return ptr, shape, dt, "ep[%s]" % base.code
        raise SimError("field %r of a value that is not an element" % e[2])

    def field(self, e, env):
        if e[1][0] == "name" and e[1][1] in env and env[e[1][1]].kind == "tuple":
            tv = env[e[1][1]]
            names = getattr(tv, "names", [])
            if e[2] in names:
                return _Val("vertex", str(names.index(e[2])), elem=tv.elem)
        ptr, shape, dt, idx = self.field_base(e, env)
        if shape == ():
            return _Val({"int": "int", "bool": "bool"}.get(dt, "scalar"), "%s[%s]" % (ptr, idx))
        out = self.new_tensor(shape)
        sz = _size(shape)
        self.emit("for (int q_ = 0; q_ < %d; ++q_) %s[q_] = %s[(long long)%s * %d + q_];"
                  % (sz, out, ptr, idx, sz))
        return _Val("tensor", out, shape)

    # indexing ---------------------------------------------------------------
    def flat(self, shape, idx):
        if len(idx) == 1 and len(shape) == 2 and 1 in shape:
            return idx[0]
        if len(idx) != len(shape):
            raise SimError("%d indices for a tensor of shape %s" % (len(idx), shape))
        code = idx[0]
        for d, i in zip(shape[1:], idx[1:]):
            code = "(%s) * %d + %s" % (code, d, i)
        return code

    def index_codes(self, args, env):
        return [self.as_scalar(self.expr(a, env), "index") for a in args]

    def read_index(self, v, args, env):
        if v.kind == "sysvec":
            return self.sysvec_read(v, args, env)
        if v.kind != "tensor":
            raise SimError("indexing a value that is not a tensor")
        if any(a[0] == "slice" for a in args):
            return self.slice(v, args, env)
        idx = self.index_codes(args, env)
        sub = self.sub_tensor(v, idx)
        if sub is not None:
            return sub
        return _Val("scalar", "%s[%s]" % (v.code, self.flat(v.shape, idx)))

    def sub_tensor(self, v, idx):
        """v(i) of a nested block (tensor[3](tensor[3](float)) is a 3x3 local
        value whose v(i) is a 3-vector): the leading indices select a
        sub-tensor, which aliases v's storage.  None when idx indexes v
        fully."""
        sh = v.shape
        if len(idx) >= len(sh) or (len(sh) == 2 and 1 in sh):
            return None
        rest = sh[len(idx):]
        off = self.flat(sh[:len(idx)], idx) if len(idx) > 1 else idx[0]
        shape = (rest[0], 1) if len(rest) == 1 else rest
        return _Val("tensor", "(%s + (%s) * %d)" % (v.code, off, _size(rest)), shape)

    def slice(self, v, args, env):
        if len(v.shape) != 2 or len(args) != 2:
            raise SimError("slices of matrices only")
        r, c = v.shape
        if args[0][0] == "slice" and args[1][0] != "slice":
            k = self.as_scalar(self.expr(args[1], env))
            return self.elementwise((r, 1), lambda q: "%s[(%s) * %d + %s]" % (v.code, q, c, k))
        if args[1][0] == "slice" and args[0][0] != "slice":
            k = self.as_scalar(self.expr(args[0], env))
            return self.elementwise((1, c), lambda q: "%s[(%s) * %d + %s]" % (v.code, k, c, q))
        return v

    # expressions ------------------------------------------------------------
    def expr(self, e, env):
        k = e[0]
        if k == "num":
            return _Val("scalar", _lit(e[1])) if e[2] else _Val("int", str(e[1]))
        if k == "bool":
            return _Val("bool", "true" if e[1] else "false")
        if k == "name":
            n = e[1]
            if n in env:
                return env[n]
            if n in self.consts:
                return self.consts[n]
            if n in self.prog["consts"]:
                ty, ce = self.prog["consts"][n]
                v = self.expr(ce, {})
                self.consts[n] = v
                return v
            raise SimError("unknown name %r" % n)
        if k == "lit":
            return self.literal(e[1], env)
        if k == "tr":
            v = self.expr(e[1], env)
            if v.kind != "tensor":
                return v
            if len(v.shape) != 2:
                raise SimError("transpose of a tensor of order %d" % len(v.shape))
            r, c = v.shape
            return self.elementwise((c, r), lambda q: "%s[(%s) %% %d * %d + (%s) / %d]"
                                    % (v.code, q, r, c, q, r))
        if k == "un":
            v = self.expr(e[2], env)
            if e[1] == "not":
                return _Val("bool", "(!(%s))" % self.as_scalar(v))
            if v.kind == "tensor":
                return self.elementwise(v.shape, lambda q: "(-%s[%s])" % (v.code, q))
            return _Val(v.kind, "(-(%s))" % v.code)
        if k == "bin":
            return self.binop(e[1], self.expr(e[2], env), self.expr(e[3], env))
        if k == "field":
            return self.field(e, env)
        if k == "call":
            return self.call(e, env)
        if k == "str":
            raise SimError("strings are not values of an element function")
        raise SimError("unsupported expression %r" % (k,))

    def literal(self, rows, env):
        if all(x[0] == "lit" for r in rows for x in r):
            rows = [s[1][0] for r in rows for s in r]     # [[..], [..]]: one row each
        shape = (len(rows), len(rows[0]))
        out = self.new_tensor(shape)
        for r, row in enumerate(rows):
            if len(row) != shape[1]:
                raise SimError("ragged tensor literal")
            for c, x in enumerate(row):
                v = self.expr(x, env)
                self.emit("%s[%d] = %s;" % (out, r * shape[1] + c, self.as_scalar(v)))
        return _Val("tensor", out, shape)

    def binop(self, op, a, b):
        if op in ("and", "or", "xor"):
            cop = {"and": "&&", "or": "||", "xor": "!="}[op]
            x, y = self.as_scalar(a), self.as_scalar(b)
            if op == "xor":
                x, y = "(bool)(%s)" % x, "(bool)(%s)" % y
            return _Val("bool", "(%s %s %s)" % (x, cop, y))
        if op in ("==", "!=", "<", ">", "<=", ">="):
            return _Val("bool", "(%s %s %s)" % (self.as_scalar(a), op, self.as_scalar(b)))
        if op == "\\":
            raise SimError("solves (\\) are not part of an element function")
        ta, tb = self.is_tensor(a), self.is_tensor(b)
        cop = {".*": "*", "./": "/"}.get(op, op)
        if not ta and not tb:
            x, y = self.as_scalar(a), self.as_scalar(b)
            if op == "^":
                return _Val("scalar", "pow((real)(%s), (real)(%s))" % (x, y))
            kind = "int" if a.kind == "int" and b.kind == "int" else "scalar"
            return _Val(kind, "(%s %s %s)" % (x, cop, y))
        if op == "*" and ta and tb:
            return self.matmul(a, b)
        if op == "^":
            raise SimError("^ of a tensor")
        if ta and tb:
            # element-wise: equal shapes, or two vectors of one length (the
            # result keeps the left one's orientation)
            vecs = (len(a.shape) == 2 and len(b.shape) == 2 and 1 in a.shape and
                    1 in b.shape and _size(a.shape) == _size(b.shape))
            if a.shape != b.shape and not vecs:
                raise SimError("%s of shapes %s and %s" % (op, a.shape, b.shape))
            return self.elementwise(a.shape, lambda q: "(%s[%s] %s %s[%s])"
                                    % (a.code, q, cop, b.code, q))
        if ta:
            s = self.as_scalar(b)
            return self.elementwise(a.shape, lambda q: "(%s[%s] %s %s)" % (a.code, q, cop, s))
        if op == "/":
            raise SimError("a scalar divided by a tensor")
        s = self.as_scalar(a)
        return self.elementwise(b.shape, lambda q: "(%s %s %s[%s])" % (s, cop, b.code, q))

    def matmul(self, a, b):
        if len(a.shape) != 2 or len(b.shape) != 2 or a.shape[1] != b.shape[0]:
            raise SimError("product of shapes %s and %s" % (a.shape, b.shape))
        (r, kk), c = a.shape, b.shape[1]
        out = self.new_tensor((r, c))
        self.emit("for (int r_ = 0; r_ < %d; ++r_)" % r)
        self.emit("  for (int c_ = 0; c_ < %d; ++c_) {" % c)
        self.emit("    real s_ = real(0);")
        self.emit("    for (int k_ = 0; k_ < %d; ++k_) s_ += %s[r_ * %d + k_] * %s[k_ * %d + c_];"
                  % (kk, a.code, kk, b.code, c))
        self.emit("    %s[r_ * %d + c_] = s_;" % (out, c))
        self.emit("  }")
        return _Val("tensor", out, (r, c))

    def call(self, e, env):
        fn, args = e[1], e[2]
        if fn[0] == "name" and fn[1] in env:
            v = env[fn[1]]
            if v.kind == "tuple":
                idx = self.as_scalar(self.expr(args[0], env), "endpoint index")
                return _Val("vertex", idx, elem=v.elem)
            return self.read_index(v, args, env)
        if fn[0] == "field":
            ptr, shape, dt, idx = self.field_base(fn, env)
            if shape == () or any(a[0] == "slice" for a in args):
                return self.read_index(self.field(fn, env), args, env)
            flat = self.flat(shape, self.index_codes(args, env))
            return _Val({"int": "int", "bool": "bool"}.get(dt, "scalar"),
                        "%s[(long long)%s * %d + %s]" % (ptr, idx, _size(shape), flat))
        if fn[0] == "call":
            return self.read_index(self.call(fn, env), args, env)
        if fn[0] != "name":
            raise SimError("unsupported call")
        name = fn[1]
        if name in self.prog["funcs"]:
            return self.user_call(self.prog["funcs"][name], [self.expr(a, env) for a in args])
        return self.builtin(name, [self.expr(a, env) for a in args])

    def builtin(self, name, args):
        if name in _MATH1 and len(args) == 1:
            return _Val("scalar", "%s((real)(%s))" % (_MATH1[name], self.as_scalar(args[0])))
        if name == "atan2" and len(args) == 2:
            return _Val("scalar", "atan2((real)(%s), (real)(%s))"
                        % (self.as_scalar(args[0]), self.as_scalar(args[1])))
        if name == "pow" and len(args) == 2:
            return self.binop("^", args[0], args[1])
        if name == "mod" and len(args) == 2:
            if args[0].kind == "int" and args[1].kind == "int":
                return _Val("int", "(%s %% %s)" % (args[0].code, args[1].code))
            return _Val("scalar", "fmod((real)(%s), (real)(%s))"
                        % (self.as_scalar(args[0]), self.as_scalar(args[1])))
        if name in ("dot", "norm", "cross"):
            vs = []
            for a in args:
                if a.kind != "tensor" or len(a.shape) != 2 or 1 not in a.shape:
                    raise SimError("%s of a value that is not a vector" % name)
                vs.append(a)
            n = _size(vs[0].shape)
            if name == "dot" and len(vs) == 2 and _size(vs[1].shape) == n:
                return _Val("scalar", self.sum_products(vs[0].code, vs[1].code, n))
            if name == "norm" and len(vs) == 1:
                return _Val("scalar", "sqrt(%s)" % self.sum_products(vs[0].code, vs[0].code, n))
            if name == "cross" and len(vs) == 2 and n == 3 and _size(vs[1].shape) == 3:
                a, b = vs[0].code, vs[1].code
                out = self.new_tensor((3, 1))
                for k in range(3):
                    i, j = (k + 1) % 3, (k + 2) % 3
                    self.emit("%s[%d] = %s[%d] * %s[%d] - %s[%d] * %s[%d];"
                              % (out, k, a, i, b, j, a, j, b, i))
                return _Val("tensor", out, (3, 1))
            raise SimError("bad arguments to %s" % name)
        if name in ("det", "inv") and len(args) == 1:
            a = args[0]
            if a.kind != "tensor" or a.shape != (3, 3):
                raise SimError("%s of a matrix that is not 3x3" % name)
            if name == "det":
                self.intrinsic("det3")
                return _Val("scalar", "simi_det3(%s)" % a.code)
            self.intrinsic("inv3")
            out = self.new_tensor((3, 3))
            self.emit("simi_inv3(%s, %s);" % (a.code, out))
            return _Val("tensor", out, (3, 3))
        raise SimError("unknown function %r" % name)

    def sum_products(self, a, b, n):
        s = self.tmp("s")
        self.emit("real %s = real(0);" % s)
        self.emit("for (int q_ = 0; q_ < %d; ++q_) %s += %s[q_] * %s[q_];" % (n, s, a, b))
        return s

    # user functions: device functions with array out-parameters
    def user_call(self, f, args, nout=1):
        name = self.helper(f, args)
        outs = []
        for rn, rty in f["results"]:
            shape = _shape_of_type(rty)
            if shape == ():
                tn = self.tmp("r")
                ct = "int" if rty[1] == "int" else "real"
                self.emit("%s %s;" % (ct, tn))
                outs.append(_Val("int" if rty[1] == "int" else "scalar", tn))
            else:
                outs.append(_Val("tensor", self.new_tensor(shape), shape))
        argc = []
        for a in args:
            if a.kind == "element":
                continue              # the helper has the map's element as `e`
            argc.append(a.code if a.kind in ("tensor", "vertex") else self.as_scalar(a))
        # every helper sees the map's element, endpoints and fields
        argc += ["e", "ep", "f"]
        self.emit("%s(%s);" % (name, ", ".join(argc + [o.code for o in outs])))
        if len(outs) != nout:
            raise SimError("%s returns %d values, %d expected" % (f["name"], len(outs), nout))
        return outs[0] if nout == 1 else outs

    def helper(self, f, args):
        done = self.st["funcs_done"]
        if f["name"] in done:
            return done[f["name"]]
        name = "simf_" + f["name"]
        done[f["name"]] = name
        if len(args) != len(f["args"]):
            raise SimError("%s takes %d arguments, %d given" % (f["name"], len(f["args"]),
                                                               len(args)))
        sub = _Gen(self.prog, self.consts, self.st)
        params, env = [], {}
        for (an, aty, _), av in zip(f["args"], args):
            if aty[0] == "element" and av.kind == "element":
                env[an] = _Val("element", "e", elem=av.elem)
                continue
            if aty[0] == "element" and av.kind == "vertex":
                # an endpoint: its local index
                params.append("int a_%s" % an)
                env[an] = _Val("vertex", "a_" + an, elem=av.elem)
                continue
            if aty[0] not in ("scalar", "tensor"):
                raise SimError("%s: only scalar, tensor and element arguments in called "
                               "functions" % f["name"])
            sh = _shape_of_type(aty)
            cn = "a_" + an
            if sh == ():
                ct = {"int": "int", "bool": "bool"}.get(aty[1], "real")
                params.append("%s %s" % (ct, cn))
                env[an] = _Val({"int": "int", "bool": "bool"}.get(aty[1], "scalar"), cn)
            else:
                if av.kind != "tensor" or _size(av.shape) != _size(sh):
                    raise SimError("%s: argument %s is not a tensor of shape %s"
                                   % (f["name"], an, sh))
                params.append("const real *%s" % cn)
                env[an] = _Val("tensor", cn, sh)
        params += ["long long e", "const int *ep", "const real *const *f"]
        sub.emit("(void)e; (void)ep; (void)f;")
        sub.vertex_map = self.vertex_map
        # results start from zero, as every local tensor does
        for rn, rty in f["results"]:
            sh = _shape_of_type(rty)
            cn = "o_" + rn
            if sh == ():
                ct = "int" if rty[1] == "int" else "real"
                params.append("%s &%s" % (ct, cn))
                env[rn] = _Val("int" if rty[1] == "int" else "scalar", cn)
                sub.emit("%s = 0;" % cn)
            else:
                params.append("real *%s" % cn)
                env[rn] = _Val("tensor", cn, sh)
                sub.emit("for (int q_ = 0; q_ < %d; ++q_) %s[q_] = real(0);" % (_size(sh), cn))
        sub.block(f["body"], env)
        src = "__device__ void %s(%s) {\n%s\n}\n" % (name, ", ".join(params),
                                                    "\n".join(sub.lines))
        self.st["funcs_out"].append(src)
        return name

    # statements -------------------------------------------------------------
    def block(self, stmts, env):
        env = dict(env)
        for s in stmts:
            self.stmt(s, env)

    def assign_tensor(self, dst, v):
        if v.kind == "tensor" and _size(v.shape) != 1:
            same = v.shape == dst.shape or (len(v.shape) == 2 and len(dst.shape) == 2 and
                                            1 in v.shape and 1 in dst.shape and
                                            _size(v.shape) == _size(dst.shape))
            if not same:
                raise SimError("assigning shape %s to %s" % (v.shape, dst.shape))
            self.emit("for (int q_ = 0; q_ < %d; ++q_) %s[q_] = %s[q_];"
                      % (_size(dst.shape), dst.code, v.code))
        else:
            self.emit("for (int q_ = 0; q_ < %d; ++q_) %s[q_] = %s;"
                      % (_size(dst.shape), dst.code, self.as_scalar(v)))

    def declare(self, name, v, env):
        cn = "v_" + name
        if v.kind == "tensor":
            self.emit("real %s[%d];" % (cn, _size(v.shape)))
            nv = _Val("tensor", cn, v.shape)
            self.assign_tensor(nv, v)
        elif v.kind in ("scalar", "int", "bool"):
            ct = {"scalar": "real", "int": "int", "bool": "bool"}[v.kind]
            self.emit("%s %s = %s;" % (ct, cn, v.code))
            nv = _Val(v.kind, cn)
        else:
            nv = v
        env[name] = nv

    def stmt(self, s, env):
        k = s[0]
        if k in ("print", "return", "nop"):
            return
        if k == "var":
            _, name, ty, init, line = s
            if ty is not None and ty[0] == "tensor":
                sh = _shape_of_type(ty)
                cn = "v_" + name
                self.emit("real %s[%d];" % (cn, _size(sh)))
                env[name] = _Val("tensor", cn, sh)
                self.assign_tensor(env[name], self.expr(init, env) if init is not None
                                   else _Val("scalar", "real(0)"))
                return
            v = self.expr(init, env) if init is not None else _Val("scalar", "real(0)")
            if ty is not None and ty[0] == "scalar":
                v = _Val({"int": "int", "bool": "bool"}.get(ty[1], "scalar"),
                         self.as_scalar(v))
            self.declare(name, v, env)
            return
        if k == "for":
            _, var, lo, hi, body, line = s
            lo_c = self.as_scalar(self.expr(lo, env))
            hi_c = self.as_scalar(self.expr(hi, env))
            cn = "i_" + var
            self.emit("for (int %s = %s; %s < %s; ++%s) {" % (cn, lo_c, cn, hi_c, cn))
            self.ind += 1
            inner = dict(env)
            inner[var] = _Val("int", cn)
            self.block(body, inner)
            self.ind -= 1
            self.emit("}")
            return
        if k == "while":
            _, cond, body, line = s
            self.emit("for (;;) {")
            self.ind += 1
            self.emit("if (!(%s)) break;" % self.as_scalar(self.expr(cond, env)))
            self.block(body, env)
            self.ind -= 1
            self.emit("}")
            return
        if k == "if":
            _, arms, els, line = s
            for n, (cond, body) in enumerate(arms):
                if n:
                    self.emit("} else {")
                    self.ind += 1
                self.emit("if (%s) {" % self.as_scalar(self.expr(cond, env)))
                self.ind += 1
                self.block(body, env)
                self.ind -= 1
            if els:
                self.emit("} else {")
                self.ind += 1
                self.block(els, env)
                self.ind -= 1
            self.emit("}")
            for _ in range(len(arms) - 1):
                self.ind -= 1
                self.emit("}")
            return
        if k == "expr":
            self.expr(s[1], env)
            return
        if k == "assign":
            self.assign(s[1], s[2], env, s[3])
            return
        if k == "massign":
            _, lhs, rhs, line = s
            if rhs[0] != "call" or rhs[1][0] != "name" or rhs[1][1] not in self.prog["funcs"]:
                raise SimError("line %d: several values are assigned from a function call "
                               "only" % line)
            f = self.prog["funcs"][rhs[1][1]]
            outs = self.user_call(f, [self.expr(a, env) for a in rhs[2]], nout=len(lhs))
            for target, v in zip(lhs, outs):
                if target[0] != "name":
                    raise SimError("line %d: unsupported assignment target" % line)
                cur = env.get(target[1])
                if cur is not None and cur.kind == "tensor":
                    self.assign_tensor(cur, v)
                elif cur is not None and cur.kind in ("scalar", "int", "bool"):
                    self.emit("%s = %s;" % (cur.code, self.as_scalar(v)))
                else:
                    self.declare(target[1], v, env)
            return
        raise SimError("line %d: %s is not part of an element function" % (s[-1], k))

    def assign(self, lhs, rhs, env, line):
        if lhs[0] == "name":
            name = lhs[1]
            if name in self.results:
                raise SimError("line %d: the whole result %r is assigned" % (line, name))
            v = self.expr(rhs, env)
            cur = env.get(name)
            if cur is not None and cur.kind == "tensor":
                self.assign_tensor(cur, v)
            elif cur is not None and cur.kind in ("scalar", "int", "bool") and \
                    not self.is_tensor(v):
                self.emit("%s = %s;" % (cur.code, self.as_scalar(v)))
            else:
                self.declare(name, v, env)
            return
        if lhs[0] == "call":
            # X(p, q)(ii, jj)(i2, j2): the index groups, outermost first
            groups, node = [], lhs
            while node[0] == "call":
                groups.append(node[2])
                node = node[1]
            groups.reverse()
            if node[0] == "name" and node[1] in self.results:
                return self.system_write(node[1], groups[0], groups[1:], rhs, env, line)
            if node[0] == "name" and node[1] in env and env[node[1]].kind == "tensor":
                v = env[node[1]]
                idx = [c for g in groups for c in self.index_codes(g, env)]
                if len(idx) < len(v.shape) and not (len(v.shape) == 2 and 1 in v.shape):
                    self.assign_tensor(self.sub_tensor(v, idx), self.expr(rhs, env))
                    return
                dst = "%s[%s]" % (v.code, self.flat(v.shape, idx))
                self.emit("%s = %s;" % (dst, self.as_scalar(self.expr(rhs, env))))
                return
        raise SimError("line %d: unsupported assignment target" % line)

    def endpoint(self, a, env, line):
        v = self.expr(a, env)
        if v.kind == "vertex":
            return v.code
        if v.kind == "element" and self.vertex_map:
            return "0"
        raise SimError("line %d: the result is indexed by endpoints v(k)" % line)

    def system_write(self, tname, idx, comps, rhs, env, line):
        """A write to the map's result: a whole block (comps empty) or a
        component chain; each write adds one term, as the lowered map adds
        it into the result (src/lower/lower_maps.cpp:38-47)."""
        if tname != self.target:      # another result of the map: not assembled here
            return
        bs = self.results[tname]
        if self.vector:
            return self.vector_write(tname, idx, comps, rhs, env, line, bs)
        if len(idx) != 2:
            raise SimError("line %d: %r is written with %d indices" % (line, tname, len(idx)))
        a, b = (self.endpoint(x, env, line) for x in idx)
        self.emit("if ((%s) == i && (%s) == j) {" % (a, b))
        self.ind += 1
        ref = "sg_term_(blk, nt_)[ck_ / %d][ck_ %% %d]" % (bs, bs)
        opn = "sg_open_term_(blk, nt_)"
        nest = self.nest
        if comps:
            cidx = [c for g in comps for c in self.index_codes(g, env)]
            v = self.expr(rhs, env)
            if nest is None and len(cidx) == 2:
                self.component_write("(%s) * %d + (%s)" % (cidx[0], bs, cidx[1]),
                                     self.as_scalar(v), opn, ref)
            elif nest is not None and len(cidx) == 4:
                nb = nest[1]
                row = "(%s) * %d + (%s)" % (cidx[0], nb, cidx[2])
                col = "(%s) * %d + (%s)" % (cidx[1], nb, cidx[3])
                self.component_write("(%s) * %d + %s" % (row, bs, col), self.as_scalar(v),
                                     opn, ref)
            elif nest is not None and len(cidx) == 2:
                # an inner block X(p, q)(ii, jj) = B (b x b); a scalar lands
                # on the inner block's entry (0, 0)
                nb = nest[1]
                self.emit("for (int u_ = 0; u_ < %d; ++u_) {" % (1 if self.is_scalar_val(v)
                                                                 else nb * nb))
                self.ind += 1
                x = self.value_at(v, "u_", nb * nb, line)
                self.component_write("((%s) * %d + u_ / %d) * %d + (%s) * %d + u_ %% %d"
                                     % (cidx[0], nb, nb, bs, cidx[1], nb, nb), x, opn, ref)
                self.ind -= 1
                self.emit("}")
            else:
                raise SimError("line %d: %d component indices for a block of %s"
                               % (line, len(cidx), "%dx%d" % (bs, bs) if nest is None else
                                  "%dx%d blocks of %dx%d" % (nest[0], nest[0], nest[1],
                                                             nest[1])))
        else:
            v = self.expr(rhs, env)
            self.emit("nt_ = sg_open_term_(blk, nt_);")
            self.emit("copen_ = 0;")
            if v.kind == "tensor" and nest is not None and len(v.shape) == 4 and \
                    _size(v.shape) == bs * bs:
                # a nested local [ii][jj][i2][j2] into the flat block
                na, nb = nest
                self.emit("for (int q_ = 0; q_ < %d; ++q_) sg_term_(blk, nt_)"
                          "[q_ / %d * %d + q_ / %d %% %d][q_ / %d %% %d * %d + q_ %% %d] += %s[q_];"
                          % (bs * bs, na * nb * nb, nb, nb, nb, nb * nb, na, nb, nb, v.code))
            elif v.kind == "tensor" and _size(v.shape) == bs * bs:
                self.emit("for (int q_ = 0; q_ < %d; ++q_) sg_term_(blk, nt_)[q_ / %d][q_ %% %d] "
                          "+= %s[q_];" % (bs * bs, bs, bs, v.code))
            elif v.kind != "tensor" or _size(v.shape) == 1:
                # a scalar written to a block lands on its entry (0, 0) alone,
                # as the lowered write `K[loc*bs*bs] += value` does (a fixed
                # point's `MD(p,p) = 1.0` in the springs programs)
                self.emit("sg_term_(blk, nt_)[0][0] += %s;" % self.as_scalar(v))
            else:
                raise SimError("line %d: a value of shape %s written to a %dx%d block"
                               % (line, v.shape if v.kind == "tensor" else (), bs, bs))
        self.ind -= 1
        self.emit("}")

    def is_scalar_val(self, v):
        return v.kind != "tensor" or _size(v.shape) == 1

    def value_at(self, v, q, n, line):
        """Entry q of an n-entry value, or the value itself if scalar."""
        if v.kind == "tensor" and _size(v.shape) == n:
            return "%s[%s]" % (v.code, q)
        if v.kind != "tensor" or _size(v.shape) == 1:
            return self.as_scalar(v)
        raise SimError("line %d: a value of shape %s written to %d entries"
                       % (line, v.shape, n))

    def component_write(self, k, x, opn, ref):
        """Component k of the block (flat index) += x.  The component joins
        the open component term unless that term already holds it;
        otherwise it opens a new term."""
        self.emit("{")
        self.ind += 1
        self.emit("const int ck_ = %s;" % k)
        self.emit("if (!copen_ || ((cmask_[ck_ >> 5] >> (ck_ & 31)) & 1u)) {")
        self.emit("  nt_ = %s;" % opn)
        self.emit("  copen_ = 1;")
        self.emit("  for (int w_ = 0; w_ < %d; ++w_) cmask_[w_] = 0;" % self.cwords)
        self.emit("}")
        self.emit("%s += %s;" % (ref, x))
        self.emit("cmask_[ck_ >> 5] |= 1u << (ck_ & 31);")
        self.ind -= 1
        self.emit("}")

    def vector_write(self, tname, idx, comps, rhs, env, line, bs):
        if len(idx) != 1:
            raise SimError("line %d: %r is written with %d indices" % (line, tname, len(idx)))
        a = self.endpoint(idx[0], env, line)
        self.emit("if ((%s) == i) {" % a)
        self.ind += 1
        ref = "sg_vterm_(vec, nt_)[ck_]"
        opn = "sg_open_vterm_(vec, nt_)"
        nest = self.nest
        if comps:
            cidx = [c for g in comps for c in self.index_codes(g, env)]
            v = self.expr(rhs, env)
            if len(cidx) == 1 and nest is None:
                self.component_write(cidx[0], self.as_scalar(v), opn, ref)
            elif len(cidx) == 2 and nest is not None:
                self.component_write("(%s) * %d + (%s)" % (cidx[0], nest[1], cidx[1]),
                                     self.as_scalar(v), opn, ref)
            elif len(cidx) == 1 and nest is not None:
                # a row x(p)(ii) = w (b entries); a scalar lands on its first
                nb = nest[1]
                self.emit("for (int u_ = 0; u_ < %d; ++u_) {" % (1 if self.is_scalar_val(v)
                                                                 else nb))
                self.ind += 1
                self.component_write("(%s) * %d + u_" % (cidx[0], nb),
                                     self.value_at(v, "u_", nb, line), opn, ref)
                self.ind -= 1
                self.emit("}")
            else:
                raise SimError("line %d: %d component indices for a vertex's %d entries"
                               % (line, len(cidx), bs))
        else:
            v = self.expr(rhs, env)
            self.emit("nt_ = sg_open_vterm_(vec, nt_);")
            self.emit("copen_ = 0;")
            if v.kind == "tensor" and _size(v.shape) == bs and \
                    (len(v.shape) == 2 and 1 in v.shape or bs == 1 or nest is not None):
                self.emit("for (int q_ = 0; q_ < %d; ++q_) sg_vterm_(vec, nt_)[q_] += %s[q_];"
                          % (bs, v.code))
            elif v.kind != "tensor" or _size(v.shape) == 1:
                # a scalar lands on the vertex's first entry alone (the
                # lowered write `f[p*bs] += value`)
                self.emit("sg_vterm_(vec, nt_)[0] += %s;" % self.as_scalar(v))
            else:
                raise SimError("line %d: a value of shape %s written to a %d-vector"
                               % (line, v.shape if v.kind == "tensor" else (), bs))
        self.ind -= 1
        self.emit("}")


# Terms: each write opens a zeroed term; past SG_TERMS the extra writes are
# summed into the last term first.
_TERM_SUPPORT = r"""
__device__ inline int sg_open_term_(sg_block *blk, int nt) {
  if (nt >= SG_TERMS) return nt + 1;
  for (int a = 0; a < BS; ++a)
    for (int b = 0; b < BS; ++b) blk[nt][a][b] = real(0);
  return nt + 1;
}
__device__ inline sg_block &sg_term_(sg_block *blk, int nt) {
  return blk[(nt < SG_TERMS ? nt : SG_TERMS) - 1];
}
"""

_VTERM_SUPPORT = r"""
__device__ inline int sg_open_vterm_(sg_vec *vec, int nt) {
  if (nt >= SG_VTERMS) return nt + 1;
  for (int a = 0; a < BS; ++a) vec[nt][a] = real(0);
  return nt + 1;
}
__device__ inline sg_vec &sg_vterm_(sg_vec *vec, int nt) {
  return vec[(nt < SG_VTERMS ? nt : SG_VTERMS) - 1];
}
"""


def _result_block(rty):
    """(block size, nesting) of a system-matrix result type.  A nested block
    tensor[a,a](tensor[b,b](T)) is stored as one (a b) x (a b) block, entry
    (ii, jj)(i2, jj2) at row ii*b + i2, column jj*b + j2; nesting is (a, b),
    None for a plain block."""
    inner = rty[2]
    if inner[0] == "scalar":
        return 1, None
    sh = _shape_of_type(inner)
    if len(sh) == 2 and sh[0] == sh[1]:
        return sh[0], None
    if len(sh) == 4 and sh[0] == sh[1] and sh[2] == sh[3]:
        return sh[0] * sh[2], (sh[0], sh[2])
    raise SimError("blocks must be square matrices or square blocks of them, not %s" % (sh,))


def _result_vector(rty):
    """(entries per vertex, nesting) of a system-vector result type: a
    nested tensor[a](tensor[b](T)) (or an a x b matrix per vertex) holds a*b
    entries, entry (ii)(jj) at ii*b + jj; nesting is (a, b), None for a
    scalar or vector per vertex."""
    inner = rty[2]
    if inner[0] == "scalar":
        return 1, None
    sh = _shape_of_type(inner)
    if len(sh) == 2 and 1 in sh:
        return _size(sh), None
    if len(sh) == 2:
        return _size(sh), sh
    raise SimError("vector results hold scalars, vectors or matrices per vertex, not %s"
                   % (sh,))


def _system_results(f):
    """{name: ("matrix" | "vector", size, nesting)} of a function's system
    results."""
    out = {}
    for rn, rty in f["results"]:
        if rty[0] != "tensor" or any(isinstance(d, int) for d in rty[1]):
            continue
        if len(rty[1]) == 2:
            out[rn] = ("matrix",) + _result_block(rty)
        elif len(rty[1]) == 1:
            out[rn] = ("vector",) + _result_vector(rty)
    return out


def compile_map(src, func, args=None, result=None):
    """The element function `func` of a map as CUDA C++ source: for a
    matrix result `element_block` (sg_jit_assembly_create), for a vector
    result `element_vector` (sg_jit_vector_create).

    args binds the map's scalar arguments by name; result names the result
    to assemble when the function has several (writes to the others are
    left out).  Returns {"source", "kind" ("matrix" | "vector"), "fields"
    [(kind, name, shape, dtype)], "card", "bs", "element", "vertex",
    "result"}: pass the field arrays in `fields` order -- element fields
    [nE * size], vertex fields [n * size]; int and bool fields as int32 /
    bool arrays.  bs is the block size (matrix) or the entries per vertex
    (vector)."""
    prog = parse(src)
    if func not in prog["funcs"]:
        raise SimError("no function %r" % func)
    f = prog["funcs"][func]
    args = dict(args or {})
    env, consts = {}, {}
    elem = vert = None
    card = None
    for an, aty, _ in f["args"]:
        if aty[0] == "scalar":
            if an not in args:
                raise SimError("map argument %r is not bound" % an)
            val = args[an]
            if aty[1] == "int":
                consts[an] = _Val("int", str(int(val)))
            elif aty[1] == "bool":
                consts[an] = _Val("bool", "true" if val else "false")
            else:
                consts[an] = _Val("scalar", _lit(val))
        elif aty[0] == "element":
            if elem is not None:
                raise SimError("two element arguments")
            elem = aty[1]
            env[an] = _Val("element", "e", elem=elem)
        elif aty[0] == "tensor" and len(aty[1]) == 1 and not isinstance(aty[1][0], int):
            # a system vector read per vertex: y(p)
            inner = aty[2]
            shape = () if inner[0] == "scalar" else _shape_of_type(inner)
            while inner[0] == "tensor":
                inner = inner[2]
            env[an] = _Val("sysvec", an, shape, elem=inner[1])
        elif aty[0] == "tuple":
            members = aty[1]
            kinds = {m[1] for m in members}
            if len(kinds) != 1:
                raise SimError("endpoint tuples of one element type only")
            vert, card = kinds.pop(), len(members)
            env[an] = _Val("tuple", None, elem=vert)
            # named members, (src : Vertex, dst : Vertex): v.src is endpoint 0
            env[an].names = [m[0] for m in members]
        else:
            raise SimError("map argument %r of type %r" % (an, aty[0]))
    if elem is None:
        raise SimError("%s takes no element" % func)
    vertex_map = card is None
    if vertex_map:
        card, vert = 1, elem
    results = _system_results(f)
    if not results:
        raise SimError("%s has no system (vertex-indexed) result" % func)
    if result is None:
        if len(results) != 1:
            raise SimError("%s has %d system results: name one" % (func, len(results)))
        result = next(iter(results))
    if result not in results:
        raise SimError("%r is not a system result of %s" % (result, func))
    kind, size, nest = results[result]
    vector = kind == "vector"
    g = _Gen(prog, consts)
    g.results = {rn: results.get(rn, (None, 0))[1] for rn, _ in f["results"]}
    g.nest = nest
    g.target = result
    g.vector = vector
    g.vertex_map = vertex_map
    g.cwords = (size * (1 if vector else size) + 31) // 32
    g.emit("int nt_ = 0, copen_ = 0;")
    g.emit("unsigned cmask_[%d] = {0};" % g.cwords)
    g.emit("(void)cmask_; (void)copen_; (void)ep;")
    g.block(f["body"], env)
    g.emit("return nt_ < %s ? nt_ : %s;" % (("SG_VTERMS",) * 2 if vector else ("SG_TERMS",) * 2))
    st = g.st
    if len(st["fields"]) > MAX_FIELDS:
        raise SimError("%s reads %d fields; the assembly takes at most %d"
                       % (func, len(st["fields"]), MAX_FIELDS))
    pre = "".join(_INTRINSICS[k] for k in st["intrinsics"]) + \
        (_VTERM_SUPPORT if vector else _TERM_SUPPORT)
    head = ("__device__ int element_vector(long long e, int i, const int *ep,"
            " const real *const *f, sg_vec *vec) {\n" if vector else
            "__device__ int element_block(long long e, int i, int j, const int *ep,"
            " const real *const *f, sg_block *blk) {\n")
    source = pre + "\n".join(st["funcs_out"]) + "\n" + head + "\n".join(g.lines) + "\n}\n"
    return {"source": source, "kind": kind, "fields": list(st["fields"]), "card": card,
            "bs": size, "element": elem, "vertex": vert, "result": result}


class SimMap:
    """A map of a `.sim` program compiled for the GPU:
    `SimMap(ctx, src, "compute_stiffness", {"h": 0.01})` parses and
    generates the element function, and NVRTC compiles it into a row-owner
    assembly (sg_jit_assembly_create; sg_jit_vector_create for a vector
    result).  assemble(mesh, fields) takes the field arrays by name --
    {"B": ..., "W": ..., "c": ...}; an element and a vertex field of the same
    name are told apart as ("element", name) / ("vertex", name) keys -- and
    returns the matrix values [nnzb * bs * bs] in the mesh's pattern, or the
    vector [n * bs]."""

    def __init__(self, ctx, src, func, args=None, result=None, dtype=None, exact=True,
                 info=None):
        import torch
        from .runtime import JitAssembly, JitVectorAssembly
        self.info = info if info is not None else compile_map(src, func, args, result)
        self.card, self.bs = self.info["card"], self.info["bs"]
        self.fields = self.info["fields"]
        cls = JitVectorAssembly if self.info["kind"] == "vector" else JitAssembly
        self.jit = cls(ctx, self.info["source"], self.card, self.bs,
                       dtype=torch.float64 if dtype is None else dtype, exact=exact)

    @classmethod
    def from_info(cls, ctx, info, dtype=None, exact=True):
        """A map from compile_map's result."""
        return cls(ctx, None, None, dtype=dtype, exact=exact, info=info)

    def field_arrays(self, fields):
        """The arrays in the generated source's order, each in its declared
        type: int fields as int32, bool as bool, float fields as floating
        point (the assembly then casts them to its dtype)."""
        import torch
        out = []
        for kind, name, shape, dt in self.fields:
            if (kind, name) in fields:
                a = fields[(kind, name)]
            elif name in fields:
                a = fields[name]
            else:
                raise SimError("field %s.%s is not given" % (kind, name))
            want = {"int": (torch.int32, np.int32), "bool": (torch.bool, np.bool_)}.get(dt)
            if isinstance(a, torch.Tensor):
                if want is not None and a.dtype != want[0]:
                    a = a.to(want[0])
                elif want is None and not a.is_floating_point():
                    a = a.double()
            else:
                a = np.asarray(a)
                if want is not None and a.dtype != want[1]:
                    a = a.astype(want[1])
                elif want is None and a.dtype.kind != "f":
                    a = a.astype(np.float64)
            out.append(a)
        return out

    def assemble(self, mesh, fields, out=None):
        if mesh.card != self.card:
            raise SimError("the mesh has %d endpoints per element, the map %d"
                           % (mesh.card, self.card))
        return self.jit.assemble(mesh, self.field_arrays(fields), out)

    def close(self):
        self.jit.close()
