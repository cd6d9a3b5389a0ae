"""Generates the reference's per-flame kernel header (flame_generated.h) for a
JSON genome, so that the reference's own chaos-game kernels
(assets/kernels/refactor.cu) can be NVRTC-compiled from their sources for a
fixed set of test flames (oracle/build_ref.py) and run beside librfk's
kernels (tests/test_gpu_refrender.py). Test infrastructure only.

Two parts, both restating the reference's host code:
  * render_template: the subset of the inja template language that
    assets/templates/flame.tpl uses (statements <# #>, expressions @ @,
    trim_blocks + lstrip_blocks, the '-' left trim of an expression), with
    the callbacks get_variation_source / get_precalc_source /
    variation_has_precalc of flame_compiler.cpp:545-566;
  * translate: the flang-to-CUDA rule table of flame_compiler.cpp:108-391
    (fma folding, aff / param / math / common members, result / p /
    weight, rand calls, vec constructors, fl:: calls, u_<name>__ locals)
    over a small recursive-descent parser of the flang subset the
    variation and common definitions use;
and the template data of flame_compiler::make_source (flame_compiler.cpp:
444-541): xform definitions keyed by structure, xform ids, the vlinks'
variations with their parameters and precalc slots, and the common values
each vlink needs, dependencies first (collect_common, :428-442).
"""
from __future__ import annotations

import re
from pathlib import Path

# ------------------------------------------------------------------ flang --
_TOK = re.compile(r"\s*(?:(\d+\.\d*|\.\d+|\d+)|([A-Za-z_][A-Za-z_0-9]*)|(:=|\+=|-=|\*=|/=|==|!=|<=|>=|&&|\|\||[-+*/()<>,;.=!{}]))")


def _tokens(src: str) -> list[tuple[str, str]]:
    out, i = [], 0
    src = src.strip()
    while i < len(src):
        m = _TOK.match(src, i)
        if not m or m.end() == i:
            if src[i:].strip() == "":
                break
            raise ValueError(f"flang: cannot tokenize at {src[i:i + 20]!r}")
        num, ident, op = m.groups()
        if num is not None:
            out.append(("dec" if "." in num else "int", num))
        elif ident is not None:
            out.append(("id", ident))
        else:
            out.append(("op", op))
        i = m.end()
    return out


class Node:
    """AST node: kind in root, scoped, assign_stmt, decl, if, break, paren,
    binop (op), unop (op), lit (dec/int/bool), member, var, call."""

    def __init__(self, kind: str, *kids, text: str = "", op: str = ""):
        self.kind, self.kids, self.text, self.op = kind, list(kids), text, op

    def walk(self):
        yield self
        for k in self.kids:
            yield from k.walk()

    def has(self, pred) -> bool:
        return any(pred(n) for n in self.walk())


class _Parser:
    def __init__(self, src: str):
        self.t = _tokens(src)
        self.i = 0

    def peek(self, k=0):
        j = self.i + k
        return self.t[j] if j < len(self.t) else ("eof", "")

    def take(self, val=None):
        tok = self.peek()
        if val is not None and tok[1] != val:
            raise ValueError(f"flang: expected {val!r}, got {tok[1]!r}")
        self.i += 1
        return tok

    def program(self) -> Node:
        stmts = []
        while self.peek()[0] != "eof":
            stmts.append(self.statement())
        return Node("root", *stmts)

    def expression_only(self) -> Node:
        e = self.expr()
        if self.peek()[1] == ";":
            self.take(";")
        if self.peek()[0] != "eof":
            raise ValueError("flang: trailing tokens")
        return e

    def statement(self) -> Node:
        tok = self.peek()
        if tok == ("id", "if"):
            self.take()
            cond = self.expr()
            then = self.statement()
            if self.peek() == ("id", "else"):
                self.take()
                return Node("if", cond, then, self.statement())
            return Node("if", cond, then)
        if tok == ("id", "break"):
            self.take()
            self.take(";")
            return Node("break")
        if tok[1] == "{":
            self.take("{")
            body = []
            while self.peek()[1] != "}":
                body.append(self.statement())
            self.take("}")
            return Node("scoped", *body)
        if tok[0] == "id" and self.peek(1)[1] == ":=":
            name = self.take()[1]
            self.take(":=")
            rhs = self.expr()
            self.take(";")
            return Node("decl", Node("var", text=name), rhs)
        e = self.assignment()
        self.take(";")
        return Node("assign_stmt", e)

    def assignment(self) -> Node:
        lhs = self.expr()
        if self.peek()[1] in ("=", "+=", "-=", "*=", "/="):
            op = self.take()[1]
            return Node("binop", lhs, self.expr(), op=op)
        return lhs

    _PREC = [("||",), ("&&",), ("==", "!="), ("<", "<=", ">", ">="), ("+", "-"), ("*", "/")]

    def expr(self, level: int = 0) -> Node:
        if level == len(self._PREC):
            return self.unary()
        lhs = self.expr(level + 1)
        while self.peek()[0] == "op" and self.peek()[1] in self._PREC[level]:
            op = self.take()[1]
            lhs = Node("binop", lhs, self.expr(level + 1), op=op)
        return lhs

    def unary(self) -> Node:
        if self.peek()[1] in ("-", "!"):
            op = self.take()[1]
            return Node("unop", self.unary(), op=op)
        return self.postfix()

    def postfix(self) -> Node:
        n = self.primary()
        while True:
            if self.peek()[1] == ".":
                self.take(".")
                n = Node("member", n, Node("var", text=self.take()[1]))
            elif self.peek()[1] == "(" and n.kind == "var":
                self.take("(")
                args = []
                while self.peek()[1] != ")":
                    args.append(self.expr())
                    if self.peek()[1] == ",":
                        self.take(",")
                self.take(")")
                n = Node("call", n, *args)
            else:
                return n

    def primary(self) -> Node:
        kind, val = self.take()
        if kind in ("dec", "int"):
            return Node("lit", text=val, op=kind)
        if kind == "id":
            if val in ("true", "false"):
                return Node("lit", text=val, op="bool")
            return Node("var", text=val)
        if val == "(":
            e = self.expr()
            self.take(")")
            return Node("paren", e)
        raise ValueError(f"flang: unexpected {val!r}")


def parse_program(src: str) -> Node:
    return _Parser(src).program()


def parse_expression(src: str) -> Node:
    return _Parser(src).expression_only()


_ASSIGN_OPS = ("=", "+=", "-=", "*=", "/=")


def _indent(s: str, ind: str = "    ") -> str:
    return "\n".join(ind + ln if ln else ln for ln in s.split("\n"))


def translate(name: str, n: Node, parent: Node | None = None, rank: int = 0) -> str:
    """create_source of flame_compiler.cpp:395-403 with the table of :108-391,
    rules tried in the table's order."""
    src = lambda k, par=n, r=0: translate(name, k, par, r)  # noqa: E731
    # fma folding of +, -, +=, -= with a product operand
    if n.kind == "binop" and n.op in ("+", "-", "+=", "-=") and any(k.kind == "binop" and k.op == "*" for k in n.kids):
        mc = 0 if (n.kids[0].kind == "binop" and n.kids[0].op == "*") else 1
        mul = n.kids[mc]
        ml, mr, add = translate(name, mul.kids[0], mul, 0), translate(name, mul.kids[1], mul, 1), \
            translate(name, n.kids[1 - mc], n, 1 - mc)
        if n.op == "+":
            return f"fl::fma<FloatT>({ml}, {mr}, {add})"
        if n.op == "-":
            return f"fl::fma<FloatT>({ml}, {mr}, -({add}))" if mc == 0 else f"fl::fma<FloatT>({ml}, -({mr}), {add})"
        if n.op == "+=":
            return f"{add} = fl::fma<FloatT>({ml}, {mr}, {add})"
        return f"{add} = fl::fma<FloatT>({ml}, -({mr}), {add})"
    # aff / param / math / common members
    if n.kind == "member" and any(k.kind == "var" and k.text in ("aff", "param", "math", "common") for k in n.kids):
        group, member = n.kids[0].text, n.kids[1].text
        if group == "aff":
            return f"aff.{member}"
        if group == "param":
            return f"p_{name}_{member}"
        if group == "math":
            return f"fl::math::{member}<FloatT>"
        return f"common_{member}"
    if n.kind in ("root", "scoped"):
        body = "\n".join(translate(name, k, n, i) for i, k in enumerate(n.kids))
        if n.kind == "root":
            if n.has(lambda x: x.kind == "break"):
                return "do {\n" + _indent(body) + "\n} while(0);"
            if n.has(lambda x: x.kind == "decl"):
                return "{\n" + _indent(body) + "\n}"
            return body
        return "{\n" + _indent(body) + "\n}"
    if n.kind == "assign_stmt":
        return src(n.kids[0]) + ";"
    if n.kind == "decl":
        lhs = f"u_{n.kids[0].text}__"
        rhs = src(n.kids[1], n, 1)
        vname = n.kids[0].text

        def assigned(x: Node) -> bool:
            if x.kind == "binop" and x.op in _ASSIGN_OPS:
                t = x.kids[0]
                return (t.kind == "var" and t.text == vname) or (t.kind == "member" and t.kids[0].kind == "var" and
                                                                 t.kids[0].text == vname)
            return False

        if parent is not None and parent.has(assigned):
            return f"auto {lhs} = {rhs};"
        return f"const auto {lhs} = {rhs};"
    if n.kind == "if":
        cond, branch = src(n.kids[0], n, 0), src(n.kids[1], n, 1)
        if n.kids[1].kind != "scoped":
            branch = "\n    " + branch
        out = f"if {cond} {branch}"
        if len(n.kids) == 3:
            el = src(n.kids[2], n, 2)
            if n.kids[2].kind not in ("scoped", "if"):
                el = "\n    " + el
            out += f"\nelse {el}"
        return out
    if n.kind == "paren":
        return f"({src(n.kids[0])})"
    if n.kind == "break":
        return "break;"
    if n.kind == "binop":
        return f"{src(n.kids[0], n, 0)} {n.op} {src(n.kids[1], n, 1)}"
    if n.kind == "unop":
        return f"{n.op}{src(n.kids[0])}"
    if n.kind == "lit":
        return f"static_cast<FloatT>({n.text})" if n.op == "dec" else n.text
    if n.kind == "member":
        return f"{src(n.kids[0], n, 0)}.{src(n.kids[1], n, 1)}"
    if n.kind == "var" and n.text in ("result", "p", "weight"):
        return {"result": "outp", "weight": f"v_{name}", "p": "inp"}[n.text]
    if n.kind == "call" and n.kids[0].text in ("rand01", "randgauss", "randbit"):
        return f"rs->{n.kids[0].text}()"
    if n.kind == "call" and n.kids[0].text in ("vec2", "vec3"):
        args = [src(k, n, i + 1) for i, k in enumerate(n.kids[1:])]
        return f"{n.kids[0].text}<FloatT>{{{', '.join(args)}}}"
    if n.kind == "call":
        fname = src(n.kids[0], n, 0)
        if len(n.kids) == 1:
            return fname + "()"
        args = ", ".join(src(k, n, i + 1) for i, k in enumerate(n.kids[1:]))
        if fname == "is_even":
            return f"fl::{fname}({args})"
        return f"fl::{fname}<FloatT>({args})"
    if n.kind == "var" and parent is not None and ((parent.kind == "call" and rank == 0) or
                                                   (parent.kind == "member" and rank == 1)):
        return n.text
    if n.kind == "var":
        return f"u_{n.text}__"
    raise ValueError(f"no rule for {n.kind}")


# --------------------------------------------------------------- database --
def _yaml_entries(text: str) -> dict[str, dict]:
    """The two shapes of config/variations_new.yml entries this harness needs:
    `name: <source>` and a block with `src:` / `precalc:` / `parameters:` /
    `tags:`; and `name: |- <multi-line source>`."""
    out: dict[str, dict] = {}
    lines = text.split("\n")
    i = 0
    while i < len(lines):
        ln = lines[i]
        m = re.match(r"^([A-Za-z_0-9]+):\s*(.*)$", ln)
        if not m:
            i += 1
            continue
        name, rest = m.group(1), m.group(2)
        block = []
        j = i + 1
        while j < len(lines) and (lines[j].startswith(" ") or lines[j].startswith("\t") or lines[j].strip() == ""):
            block.append(lines[j])
            j += 1
        entry: dict = {"src": None, "precalc": None, "parameters": [], "precalc_params": []}
        if rest and rest not in ("|-", "|"):
            entry["src"] = rest
        elif rest in ("|-", "|"):
            entry["src"] = "\n".join(b.strip() for b in block)
        else:
            k = 0
            while k < len(block):
                b = block[k]
                mm = re.match(r"^\s*(src|precalc|parameters|tags):\s*(.*)$", b)
                if not mm:
                    k += 1
                    continue
                key, val = mm.group(1), mm.group(2)
                sub = []
                k += 1
                base = len(b) - len(b.lstrip())
                while k < len(block) and (block[k].strip() == "" or len(block[k]) - len(block[k].lstrip()) > base):
                    sub.append(block[k])
                    k += 1
                if key in ("src", "precalc"):
                    entry[key] = "\n".join(s.strip() for s in sub) if val in ("|-", "|", "") else val
                elif key == "parameters":
                    for s in sub:
                        pm = re.match(r"^\s*([A-Za-z_0-9]+):\s*(.*)$", s)
                        if pm and len(s) - len(s.lstrip()) == base + 2:
                            entry["parameters"].append(pm.group(1))
                            if "precalc" in pm.group(2):
                                entry["precalc_params"].append(pm.group(1))
        out[name] = entry
        i = j
    return out


class RefDatabase:
    """Variation and common definitions of the reference's config directory."""

    def __init__(self, config_dir: Path):
        self.variations = _yaml_entries((config_dir / "variations_new.yml").read_text())
        self.common = {k: v["src"] for k, v in _yaml_entries((config_dir / "common.yml").read_text()).items()}
        self._vsrc: dict[str, tuple[str, str]] = {}

    def apply_ast(self, name: str) -> Node:
        return parse_program(self.variations[name]["src"])

    def parameters(self, name: str) -> tuple[list[str], list[str]]:
        """(ordinary, precalc) parameter names, sorted as the reference's map."""
        e = self.variations[name]
        pre = sorted(e["precalc_params"])
        return sorted(p for p in e["parameters"] if p not in pre), pre

    def variation_source(self, name: str) -> tuple[str, str]:
        if name not in self._vsrc:
            e = self.variations[name]
            apply = translate(name, parse_program(e["src"]))
            pre = translate(name, parse_program(e["precalc"])) if e.get("precalc") else ""
            self._vsrc[name] = (apply, pre)
        return self._vsrc[name]

    def collect_common(self, ast: Node, storage: list[str]) -> None:
        for n in ast.walk():
            if n.kind == "member" and n.kids[0].kind == "var" and n.kids[0].text == "common":
                cname = n.kids[1].text
                if cname in storage:
                    continue
                self.collect_common(parse_expression(self.common[cname]), storage)
                storage.append(cname)

    def common_source(self, cname: str) -> str:
        return translate(cname, parse_expression(self.common[cname]))


# ---------------------------------------------------------------- template --
class _Obj(dict):
    def __getattr__(self, k):
        try:
            v = self[k]
        except KeyError as e:
            raise AttributeError(k) from e
        return _wrap(v)


def _wrap(v):
    if isinstance(v, dict) and not isinstance(v, _Obj):
        return _Obj(v)
    return v


def _render_value(v) -> str:
    if isinstance(v, bool):
        return "true" if v else "false"
    return str(v)


_STMT = re.compile(r"<#(.*?)#>", re.S)
_EXPR = re.compile(r"@(-?)([^@\n]*?)@")


def _tokenize_template(text: str) -> list[tuple[str, str]]:
    """Text / statement / expression pieces with trim_blocks and
    lstrip_blocks applied around statements, and '@-' trimming the
    whitespace before an expression on its line."""
    pieces: list[tuple[str, str]] = []
    pos = 0
    for m in _STMT.finditer(text):
        pieces.append(("text", text[pos:m.start()]))
        pieces.append(("stmt", m.group(1).strip()))
        pos = m.end()
    pieces.append(("text", text[pos:]))
    # lstrip: spaces / tabs from the line start up to a statement; trim: the
    # first newline after a statement
    for i, (kind, val) in enumerate(pieces):
        if kind != "stmt":
            continue
        if i > 0 and pieces[i - 1][0] == "text":
            prev = pieces[i - 1][1]
            nl = prev.rfind("\n")
            tail = prev[nl + 1:]
            if tail.strip(" \t") == "":
                pieces[i - 1] = ("text", prev[:nl + 1])
        if i + 1 < len(pieces) and pieces[i + 1][0] == "text":
            nxt = pieces[i + 1][1]
            if nxt.startswith("\n"):
                pieces[i + 1] = ("text", nxt[1:])
            elif nxt.startswith("\r\n"):
                pieces[i + 1] = ("text", nxt[2:])
    out: list[tuple[str, str]] = []
    for kind, val in pieces:
        if kind == "stmt":
            out.append((kind, val))
            continue
        p = 0
        for m in _EXPR.finditer(val):
            before = val[p:m.start()]
            if m.group(1) == "-":
                nl = before.rfind("\n")
                if before[nl + 1:].strip(" \t") == "":
                    before = before[:nl + 1]
            out.append(("text", before))
            out.append(("expr", m.group(2).strip()))
            p = m.end()
        out.append(("text", val[p:]))
    return out


def _to_python(expr: str) -> str:
    e = re.sub(r"\bnot\b", " not ", expr)
    return e


def render_template(text: str, data: dict, callbacks: dict) -> str:
    pieces = _tokenize_template(text)

    # block structure
    def build(i: int, stop: tuple[str, ...]):
        nodes = []
        while i < len(pieces):
            kind, val = pieces[i]
            if kind == "stmt":
                head = val.split()[0]
                if head in stop:
                    return nodes, i
                if head == "for":
                    body, j = build(i + 1, ("endfor",))
                    nodes.append(("for", val, body))
                    i = j + 1
                    continue
                if head == "if":
                    body, j = build(i + 1, ("else", "endif"))
                    other = []
                    if pieces[j][1].split()[0] == "else":
                        other, j = build(j + 1, ("endif",))
                    nodes.append(("if", val, body, other))
                    i = j + 1
                    continue
                if head == "set":
                    nodes.append(("set", val))
                    i += 1
                    continue
                raise ValueError(f"template statement {val!r}")
            nodes.append((kind, val))
            i += 1
        return nodes, i

    tree, _ = build(0, ())

    def ev(expr: str, scope: dict):
        env = {"length": len, "join": lambda a, s: s.join(_render_value(x) for x in a),
               "at": lambda o, k: _wrap(o[k] if not isinstance(o, dict) else o[str(k)] if str(k) in o else o[k]),
               "range": range, **callbacks}
        env.update({k: _wrap(v) for k, v in scope.items()})
        return eval(_to_python(expr), {"__builtins__": {}}, env)  # noqa: S307 (template of the reference)

    def run(nodes, scope) -> str:
        out = []
        for nd in nodes:
            if nd[0] == "text":
                out.append(nd[1])
            elif nd[0] == "expr":
                out.append(_render_value(ev(nd[1], scope)))
            elif nd[0] == "set":
                m = re.match(r"set\s+(\w+)\s*=\s*(.*)$", nd[1])
                scope[m.group(1)] = ev(m.group(2), scope)
            elif nd[0] == "if":
                out.append(run(nd[2] if ev(nd[1][2:].strip(), scope) else nd[3], scope))
            elif nd[0] == "for":
                m = re.match(r"for\s+(\w+)(?:\s*,\s*(\w+))?\s+in\s+(.*)$", nd[1])
                a, b, seq = m.group(1), m.group(2), ev(m.group(3), scope)
                items = list(seq.items()) if isinstance(seq, dict) else list(seq)
                for idx, it in enumerate(items):
                    inner = dict(scope)
                    if b:
                        inner[a], inner[b] = it
                    else:
                        inner[a] = it
                    inner["loop"] = {"index": idx, "is_last": idx == len(items) - 1, "is_first": idx == 0}
                    out.append(run(nd[2], inner))
        return "".join(out)

    return run(tree, dict(data))


# -------------------------------------------------------------- the header --
def _structure_key(xf: dict) -> str:
    """A name for the xform's structure (flame_compiler.cpp keys its
    definitions by xform::hash, the variation names per vlink)."""
    parts = ["_".join(sorted(vl["variations"])) for vl in xf["vchain"]]
    return "S" + "__".join(parts)


def _type_name(key: str, table: dict) -> str:
    if key not in table:
        table[key] = f"x{len(table)}"
    return table[key]


def template_data(db: RefDatabase, g: dict, affine_indices: list[int]) -> tuple[dict, dict]:
    """make_source's data for the genome and the translated variation sources."""
    xforms = list(g["xforms"]) + ([g["final_xform"]] if "final_xform" in g else [])
    names: dict[str, str] = {}
    defs: dict[str, dict] = {}
    ids = []
    needed: set[str] = set()
    for i, xf in enumerate(xforms):
        h = _type_name(_structure_key(xf), names)
        ids.append({"hash": h, "id": "final" if i == len(g["xforms"]) else str(i)})
        if h in defs:
            continue
        vchain = []
        for vl in xf["vchain"]:
            vars_, common = [], []
            for name in sorted(vl["variations"]):
                if name not in db.variations:
                    raise ValueError(f"unknown variation {name}")
                par, pre = db.parameters(name)
                vars_.append({"name": name, "parameters": par, "precalc": pre})
                db.collect_common(db.apply_ast(name), common)
                needed.add(name)
            vchain.append({"variations": vars_,
                           "common": [{"name": c, "source": db.common_source(c)} for c in common]})
        defs[h] = {"vchain": vchain}
    info = {"xform_definitions": dict(sorted(defs.items())), "xforms": ids,
            "num_standard_xforms": len(g["xforms"]), "use_chaos": "chaos" in g,
            "affine_indices": list(affine_indices)}
    sources = {v: db.variation_source(v) for v in needed}
    return info, sources


def flame_header(reference_root: Path, g: dict, affine_indices: list[int]) -> str:
    db = RefDatabase(reference_root / "config")
    info, sources = template_data(db, g, affine_indices)

    def expand(src: str, ind: str) -> str:
        return "\n".join(ind + ln for ln in src.split("\n"))

    cbs = {"get_variation_source": lambda n, ind: expand(sources[n][0], ind),
           "get_precalc_source": lambda n, ind: expand(sources[n][1], ind),
           "variation_has_precalc": lambda n: bool(sources[n][1])}
    return render_template((reference_root / "assets" / "templates" / "flame.tpl").read_text(), info, cbs)
