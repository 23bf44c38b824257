"""Mechanical Rust -> C++ translation of fluid-toy's host-side functions on
the SPH step's path.

TEST INFRASTRUCTURE ONLY. The reference computes the step's parameter
structs, integrates its rigid body and spawns particles in Rust on the CPU
(src/state/simulation.rs, src/state/rigid_body.rs,
src/simulation/particle.rs, src/simulation/sph_3d_grid.rs). No Rust
toolchain exists here, so this script reads those files where they lie and
emits C++ with the same statements in the same order, so that the
reference's own host arithmetic can run and pin the library's restatement
(fluid-toy_gb300/csrc/host_params.cpp, rigid_math.h, fs_spawn_positions).
Its output goes only to oracle/_ref/ (never committed).

The translation covers the Rust subset those functions use: structs with
named fields, C-like enums, impl blocks (methods become free functions
m_<name>(self, ...), associated functions <Type>__<name>(...)), let with
identifier / tuple / array patterns, if / for / match as statements and
expressions, ranges, struct and array literals, `as` casts, and the float
methods and iterator adapters listed in rs_runtime.hpp, which gives each its
Rust meaning. Every expression is emitted fully parenthesised, so Rust's
precedence and left-to-right grouping carry over; compiled with
-ffp-contract=off, like rustc (LLVM fuses nothing without fast-math flags).
"""
from __future__ import annotations

import re
from dataclasses import dataclass, field

TOKEN_RE = re.compile(r"""
    (?P<ws>\s+)
  | (?P<comment>//[^\n]*)
  | (?P<str>b?"(?:[^"\\]|\\.)*")
  | (?P<rawstr>r\#*")
  | (?P<char>'(?:[^'\\\n]|\\.[^']*)')
  | (?P<lifetime>'[A-Za-z_]\w*)
  | (?P<num>(?:\d[\d_]*\.(?!\.)[\d_]*|\d[\d_]*)(?:[eE][+-]?\d+)?(?:f32|f64|u8|u16|u32|u64|usize|i8|i16|i32|i64|isize)?)
  | (?P<id>[A-Za-z_]\w*)
  | (?P<op>::|->|=>|\.\.=|\.\.|==|!=|<=|>=|&&|\|\||\+=|-=|\*=|/=|%=|<<|>>|[-+*/%&|^!~<>=(){}\[\];:,.?\#@$])
""", re.X)


@dataclass
class Tok:
    kind: str
    text: str


def tokenize(src: str) -> list[Tok]:
    out: list[Tok] = []
    pos, n = 0, len(src)
    while pos < n:
        if src.startswith("/*", pos):  # nested block comments
            depth, pos = 1, pos + 2
            while depth and pos < n:
                if src.startswith("/*", pos):
                    depth, pos = depth + 1, pos + 2
                elif src.startswith("*/", pos):
                    depth, pos = depth - 1, pos + 2
                else:
                    pos += 1
            continue
        m = TOKEN_RE.match(src, pos)
        if not m:
            raise SyntaxError(f"cannot tokenize near: {src[pos:pos + 40]!r}")
        kind = m.lastgroup
        if kind == "rawstr":
            hashes = m.group(kind).count("#")
            end = src.index('"' + "#" * hashes, m.end())
            pos = end + 1 + hashes
            out.append(Tok("str", '""'))
            continue
        pos = m.end()
        if kind in ("ws", "comment"):
            continue
        out.append(Tok(kind, m.group(kind)))
    return out


# ---- types ---------------------------------------------------------------------
PRIM = {"f32": "float", "f64": "double", "u8": "uint8_t", "u16": "uint16_t", "u32": "uint32_t",
        "u64": "uint64_t", "usize": "size_t", "i8": "int8_t", "i16": "int16_t", "i32": "int32_t",
        "i64": "int64_t", "isize": "ptrdiff_t", "bool": "bool"}


@dataclass
class FnItem:
    name: str
    owner: str | None          # impl type, or None for a free function
    params: list               # [(name, cpp type)] (self excluded)
    self_kind: str | None      # None, "ref", "mut"
    ret: str                   # cpp return type ("void" if none)
    body: list[Tok]


@dataclass
class StructItem:
    name: str
    fields: list               # [(name, cpp type)]


@dataclass
class EnumItem:
    name: str
    variants: list             # [(name, value)]


@dataclass
class Module:
    structs: dict = field(default_factory=dict)
    enums: dict = field(default_factory=dict)
    fns: dict = field(default_factory=dict)      # key: name or Owner::name


class Parser:
    """Items of one Rust file: structs, enums, free functions and impl blocks;
    everything else is skipped by balanced brackets."""

    def __init__(self, toks: list[Tok]):
        self.t = toks
        self.i = 0

    def peek(self, k: int = 0) -> Tok | None:
        j = self.i + k
        return self.t[j] if j < len(self.t) else None

    def next(self) -> Tok:
        tok = self.t[self.i]
        self.i += 1
        return tok

    def expect(self, text: str) -> Tok:
        tok = self.next()
        if tok.text != text:
            raise SyntaxError(f"expected {text!r}, got {tok.text!r} at token {self.i}")
        return tok

    def skip_balanced(self, open_: str, close: str) -> list[Tok]:
        self.expect(open_)
        depth, out = 1, []
        while True:
            tok = self.next()
            if tok.text == open_:
                depth += 1
            elif tok.text == close:
                depth -= 1
                if depth == 0:
                    return out
            out.append(tok)

    def skip_angles(self):
        """Skip a generic argument list starting at '<' (">>" closes two)."""
        depth = 0
        while True:
            t = self.next().text
            depth += t.count("<") if t in ("<", "<<") else 0
            depth -= {">": 1, ">>": 2}.get(t, 0)
            if depth <= 0:
                return

    def skip_attrs_and_vis(self):
        while True:
            tok = self.peek()
            if tok is None:
                return
            if tok.text == "#":
                self.next()
                if self.peek().text == "!":
                    self.next()
                self.skip_balanced("[", "]")
            elif tok.text == "pub":
                self.next()
                if self.peek().text == "(":
                    self.skip_balanced("(", ")")
            else:
                return

    def type_(self, self_type: str | None = None) -> str:
        tok = self.next()
        if tok.text == "&":
            if self.peek().kind == "lifetime":
                self.next()
            if self.peek().text == "mut":
                self.next()
                return self.type_(self_type) + "&"
            return "const " + self.type_(self_type) + "&"
        if tok.text == "[":
            inner = self.type_(self_type)
            if self.peek().text == ";":
                self.next()
                n = []
                while self.peek().text != "]":
                    n.append(self.next().text)
                self.expect("]")
                return f"std::array<{inner}, {''.join(n)}>"
            self.expect("]")
            return f"rs::Slice<{inner}>"
        if tok.text == "(":
            parts = []
            while self.peek().text != ")":
                parts.append(self.type_(self_type))
                if self.peek().text == ",":
                    self.next()
            self.expect(")")
            return f"std::tuple<{', '.join(parts)}>" if parts else "void"
        path = [tok.text]
        while self.peek() is not None and self.peek().text == "::":
            self.next()
            path.append(self.next().text)
        if self.peek() is not None and self.peek().text == "<":  # generics: not translated
            self.skip_angles()
            return "rs::Opaque"
        name = path[-1]
        if name == "Self" and self_type:
            return self_type
        if name in PRIM:
            return PRIM[name]
        if len(path) > 1 and path[0] == "wgpu":
            return f"rs::wgpu_{name}"
        return name

    def fn_item(self, owner: str | None) -> FnItem:
        self.expect("fn")
        name = self.next().text
        if self.peek().text == "<":
            self.skip_angles()
        self.expect("(")
        params, self_kind = [], None
        while self.peek().text != ")":
            if self.peek().text == "&" and self.peek(1).text in ("self", "mut"):
                self.next()
                if self.peek().text == "mut":
                    self.next()
                    self_kind = "mut"
                else:
                    self_kind = "ref"
                self.expect("self")
            elif self.peek().text == "self":
                self.next()
                self_kind = "val"
            elif self.peek().text == "mut" and self.peek(1).text == "self":
                self.next()
                self.next()
                self_kind = "val"
            else:
                if self.peek().text == "mut":
                    self.next()
                pname = self.next().text
                self.expect(":")
                params.append((pname, self.type_(owner)))
            if self.peek().text == ",":
                self.next()
        self.expect(")")
        ret = "void"
        if self.peek().text == "->":
            self.next()
            ret = self.type_(owner)
        if self.peek().text == "where":
            while self.peek().text != "{":
                self.next()
        body = self.skip_balanced("{", "}")
        return FnItem(name, owner, params, self_kind, ret, body)

    def module(self) -> Module:
        m = Module()
        while self.peek() is not None:
            self.skip_attrs_and_vis()
            tok = self.peek()
            if tok is None:
                break
            if tok.text == "struct":
                self.next()
                name = self.next().text
                if self.peek().text == "{":
                    body = Parser(self.skip_balanced("{", "}"))
                    fields = []
                    while body.peek() is not None:
                        body.skip_attrs_and_vis()
                        if body.peek() is None:
                            break
                        fname = body.next().text
                        body.expect(":")
                        fields.append((fname, body.type_(name)))
                        if body.peek() is not None and body.peek().text == ",":
                            body.next()
                    m.structs[name] = StructItem(name, fields)
                else:
                    while self.next().text != ";":
                        pass
            elif tok.text == "enum":
                self.next()
                name = self.next().text
                body = Parser(self.skip_balanced("{", "}"))
                variants, value = [], 0
                while body.peek() is not None:
                    body.skip_attrs_and_vis()
                    if body.peek() is None:
                        break
                    vname = body.next().text
                    if body.peek() is not None and body.peek().text == "=":
                        body.next()
                        value = int(body.next().text.replace("_", ""))
                    if body.peek() is not None and body.peek().text in ("(", "{"):
                        opener = body.peek().text
                        body.skip_balanced(opener, ")" if opener == "(" else "}")
                        variants = None  # data-carrying variants: not translatable
                        break
                    variants.append((vname, value))
                    value += 1
                    if body.peek() is None:
                        break
                    if body.peek() is not None and body.peek().text == ",":
                        body.next()
                if variants is not None:
                    m.enums[name] = EnumItem(name, variants)
            elif tok.text == "impl":
                self.next()
                if self.peek().text == "<":
                    self.skip_angles()
                head = []
                while self.peek().text != "{":
                    if self.peek().text == "<":
                        self.skip_angles()
                        continue
                    head.append(self.next().text)
                trait = "for" in head
                after = head[head.index("for") + 1:] if trait else head
                owner = [x for x in after if x not in ("::",)][-1]
                inner = Parser(self.skip_balanced("{", "}"))
                while inner.peek() is not None:
                    inner.skip_attrs_and_vis()
                    if inner.peek() is None:
                        break
                    while inner.peek().text in ("const", "unsafe", "async") and \
                            inner.peek(1).text in ("fn", "unsafe", "async"):
                        inner.next()
                    if inner.peek().text == "fn":
                        f = inner.fn_item(owner)
                        if not trait:
                            m.fns[f"{owner}::{f.name}"] = f
                    elif inner.peek().text in ("const", "type"):
                        while inner.next().text != ";":
                            pass
                    else:
                        raise SyntaxError(f"impl {owner}: unexpected {inner.peek().text!r}")
            elif tok.text in ("const", "unsafe", "async") and self.peek(1).text in ("fn", "unsafe"):
                self.next()
            elif tok.text == "fn":
                f = self.fn_item(None)
                m.fns[f.name] = f
            elif tok.text == "mod":
                self.next()
                self.next()
                if self.peek().text == "{":
                    self.skip_balanced("{", "}")
                else:
                    self.expect(";")
            elif tok.text in ("use", "const", "static", "type"):
                depth = 0
                while True:  # to the ';' that ends the item
                    t = self.next().text
                    depth += t in ("{", "(", "[")
                    depth -= t in ("}", ")", "]")
                    if t == ";" and depth == 0:
                        break
            elif tok.text in ("trait",):
                while self.peek().text != "{":
                    self.next()
                self.skip_balanced("{", "}")
            else:
                raise SyntaxError(f"unexpected top-level token {tok.text!r}")
        return m


# ---- function bodies -------------------------------------------------------------
BINARY = [  # (operators, precedence); higher binds tighter
    (("||",), 1), (("&&",), 2), (("==", "!=", "<", ">", "<=", ">="), 3), (("|",), 4),
    (("^",), 5), (("&",), 6), (("<<", ">>"), 7), (("+", "-"), 8), (("*", "/", "%"), 9),
]
PREC = {op: p for ops, p in BINARY for op in ops}
AS_PREC = 10
ASSIGN = {"=", "+=", "-=", "*=", "/=", "%="}
FLOAT_METHODS = {"sqrt", "abs", "ceil", "floor", "sin", "cos", "tan", "exp", "ln", "sin_cos",
                 "powi", "powf", "min", "max", "round", "signum", "clamp", "atan2", "to_radians"}


class Body:
    """Translates one function body (tokens) into C++ statements."""

    def __init__(self, toks: list[Tok], env: "Translator", owner: str | None):
        self.t = toks
        self.i = 0
        self.env = env
        self.owner = owner
        self.refs: set[str] = set()  # names bound to references (loop variables)
        self.tmp = 0

    # token helpers
    def peek(self, k: int = 0) -> Tok | None:
        j = self.i + k
        return self.t[j] if j < len(self.t) else None

    def at(self, text: str, k: int = 0) -> bool:
        tok = self.peek(k)
        return tok is not None and tok.text == text

    def next(self) -> Tok:
        tok = self.t[self.i]
        self.i += 1
        return tok

    def expect(self, text: str) -> Tok:
        tok = self.next()
        if tok.text != text:
            raise SyntaxError(f"expected {text!r}, got {tok.text!r}")
        return tok

    def fresh(self, base: str) -> str:
        self.tmp += 1
        return f"_{base}{self.tmp}"

    # blocks and statements
    def block_stmts(self, value: str | None) -> list[str]:
        """Statements of a `{ ... }` block (current token '{'). A trailing
        expression becomes `<value> expr;` ("return" in a function body), or
        is evaluated and dropped when value is None."""
        self.expect("{")
        out: list[str] = []
        while not self.at("}"):
            out.extend(self.statement(value))
        self.expect("}")
        return out

    def statement(self, value: str | None) -> list[str]:
        tok = self.peek()
        if tok.text == ";":
            self.next()
            return []
        if tok.text == "let":
            return self.let_stmt()
        if tok.text == "return":
            self.next()
            if self.at(";"):
                self.next()
                return ["return;"]
            e = self.expr()
            self.expect(";")
            return [f"return {e};"]
        if tok.text in ("continue", "break"):
            self.next()
            self.expect(";")
            return [f"{tok.text};"]
        if tok.text == "for":
            return self.for_stmt()
        if tok.text == "while":
            self.next()
            cond = self.expr(no_struct=True)
            return [f"while ({cond}) {{", *self.block_stmts(None), "}"]
        if tok.text == "if":
            stmts = self.if_stmt(value)
            return stmts
        if tok.text == "match":
            return self.match_stmt(value)
        if tok.text == "{":
            return ["{", *self.block_stmts(value), "}"]
        lhs = self.expr()
        if self.peek() is not None and self.peek().text in ASSIGN:
            op = self.next().text
            rhs = self.expr()
            self.expect(";")
            return [f"{lhs} {op} {rhs};"]
        if self.at(";"):
            self.next()
            return [f"{lhs};"]
        if self.at("}"):  # trailing expression
            if value is None:
                return [f"(void)({lhs});"]
            return [f"{value} {lhs};"]
        raise SyntaxError(f"unexpected {self.peek().text!r} after expression {lhs}")

    def pattern(self) -> tuple[str, list[str]]:
        """A let / for pattern: (binding text, names)."""
        if self.at("mut"):
            self.next()
        if self.at("("):
            self.next()
            names = []
            while not self.at(")"):
                names.append(self.pattern()[0])
                if self.at(","):
                    self.next()
            self.expect(")")
            return "[" + ", ".join(names) + "]", names
        if self.at("["):
            self.next()
            names = []
            while not self.at("]"):
                names.append(self.pattern()[0])
                if self.at(","):
                    self.next()
            self.expect("]")
            return "[" + ", ".join(names) + "]", names
        if self.at("&"):
            self.next()
            return self.pattern()
        name = self.next().text
        return name, [name]

    def let_stmt(self) -> list[str]:
        self.expect("let")
        binding, names = self.pattern()
        ty = None
        if self.at(":"):
            self.next()
            p = Parser(self.t)
            p.i = self.i
            ty = p.type_(self.owner)
            self.i = p.i
        if not self.at("="):
            self.expect(";")
            return [f"{ty or 'auto'} {binding}{{}};"]
        self.next()
        e = self.expr()
        self.expect(";")
        if binding.startswith("["):
            return [f"auto {binding} = {e};"]
        return [f"{ty or 'auto'} {binding} = {e};"]

    def for_stmt(self) -> list[str]:
        self.expect("for")
        binding, names = self.pattern()
        # remember whether the pattern was (a, &b)
        self.expect("in")
        start = self.i
        # range?
        depth, j = 0, self.i
        is_range = False
        while j < len(self.t):
            tx = self.t[j].text
            if tx in ("(", "[") or (tx == "{" and depth > 0):
                depth += 1
            elif tx in (")", "]") or (tx == "}" and depth > 0):
                depth -= 1
            elif tx == "{" and depth == 0:
                break
            elif tx in ("..", "..=") and depth == 0:
                is_range = True
            j += 1
        if is_range:
            lo = self.expr(stop_range=True, no_struct=True)
            op = self.next().text
            hi = self.expr(no_struct=True)
            var = names[0]
            end = self.fresh("end")
            cmp = "<=" if op == "..=" else "<"
            return ["{", f"const auto {end} = {hi};",
                    f"for (auto {var} = static_cast<std::remove_cvref_t<decltype({end})>>({lo}); "
                    f"{var} {cmp} {end}; ++{var}) {{", *self.block_stmts(None), "}", "}"]
        # `&mut a`, `&a`, `a.iter()`, `a.iter_mut()`, `a.iter_mut().zip(&b)`
        mut = False
        if self.at("&"):
            self.next()
            if self.at("mut"):
                self.next()
                mut = True
        src = self.expr(no_struct=True, raw_iter=True)
        if isinstance(src, tuple):  # zip
            a, b = src
            k = self.fresh("k")
            na, nb = names
            self.refs.add(na)
            return [f"for (size_t {k} = 0; {k} < std::min(({a}).size(), ({b}).size()); ++{k}) {{",
                    f"auto &{na} = ({a})[{k}];", f"const auto {nb} = ({b})[{k}];",
                    *self.block_stmts(None), "}"]
        var = names[0]
        self.refs.add(var)
        qual = "auto &" if mut or src.endswith("/*iter_mut*/") else "const auto &"
        src = src.replace("/*iter_mut*/", "").replace("/*iter*/", "")
        return [f"for ({qual}{var} : {src}) {{", *self.block_stmts(None), "}"]

    def if_stmt(self, value: str | None) -> list[str]:
        self.expect("if")
        cond = self.expr(no_struct=True)
        out = [f"if ({cond}) {{", *self.block_stmts(value), "}"]
        if self.at("else"):
            self.next()
            if self.at("if"):
                rest = self.if_stmt(value)
                out[-1] = "} else " + rest[0]
                out.extend(rest[1:])
            else:
                out[-1] = "} else {"
                out.extend(self.block_stmts(value))
                out.append("}")
        return out

    def match_arms(self):
        """(patterns, arm tokens handled by callback) for the current match."""
        self.expect("{")
        arms = []
        while not self.at("}"):
            pats = [self.path_text()]
            while self.at("|"):
                self.next()
                pats.append(self.path_text())
            self.expect("=>")
            if self.at("{"):
                start = self.i
                depth = 0
                while True:
                    tx = self.next().text
                    depth += tx == "{"
                    depth -= tx == "}"
                    if depth == 0:
                        break
                arms.append((pats, self.t[start:self.i], True))
            else:
                start = self.i
                depth = 0
                while True:
                    tx = self.peek().text
                    if depth == 0 and tx in (",", "}"):
                        break
                    depth += tx in ("(", "[", "{")
                    depth -= tx in (")", "]", "}")
                    self.next()
                arms.append((pats, self.t[start:self.i], False))
            if self.at(","):
                self.next()
        self.expect("}")
        return arms

    def path_text(self) -> str:
        parts = [self.next().text]
        while self.at("::"):
            self.next()
            if self.at("<"):  # turbofish: keep the type argument
                self.next()
                p = Parser(self.t)
                p.i = self.i
                targ = p.type_(self.owner)
                self.i = p.i
                self.expect(">")
                parts[-1] += f"<{targ}>"
                continue
            parts.append(self.next().text)
        if parts == ["Self"] or (parts[0] == "Self" and self.owner):
            parts[0] = self.owner
        return "::".join(parts)

    def match_code(self, scrut: str, arms, value: str | None) -> list[str]:
        out = []
        first = True
        for pats, toks, is_block in arms:
            conds = [f"({scrut}) == {p}" for p in pats if p != "_"]
            head = ("if" if first else "} else if") + f" ({' || '.join(conds)}) {{"
            if not conds:
                head = "{" if first else "} else {"
            out.append(head)
            sub = Body(toks, self.env, self.owner)
            sub.refs = set(self.refs)
            sub.tmp = self.tmp + 100
            if is_block:
                out.extend(sub.block_stmts(value))
            else:
                e = sub.expr()
                out.append(f"{value} {e};" if value else f"(void)({e});")
            first = False
        out.append("}")
        return out

    def match_stmt(self, value: str | None) -> list[str]:
        self.expect("match")
        scrut = self.expr(no_struct=True)
        return self.match_code(scrut, self.match_arms(), value)

    # expressions ------------------------------------------------------------------
    def expr(self, min_prec: int = 0, no_struct: bool = False, stop_range: bool = False,
             raw_iter: bool = False):
        lhs = self.unary(no_struct, raw_iter)
        if isinstance(lhs, tuple):
            return lhs
        while True:
            tok = self.peek()
            if tok is None:
                return lhs
            if tok.text == "as":
                if AS_PREC < min_prec:
                    return lhs
                self.next()
                p = Parser(self.t)
                p.i = self.i
                ty = p.type_(self.owner)
                self.i = p.i
                lhs = f"rs::as<{ty}>({lhs})"
                continue
            if stop_range and tok.text in ("..", "..="):
                return lhs
            prec = PREC.get(tok.text)
            if prec is None or prec < min_prec or (tok.kind != "op"):
                return lhs
            self.next()
            rhs = self.expr(prec + 1, no_struct, stop_range)
            lhs = f"({lhs} {tok.text} {rhs})"

    def unary(self, no_struct: bool, raw_iter: bool = False):
        tok = self.peek()
        if tok.text == "-":
            self.next()
            return f"(-{self.unary(no_struct)})"
        if tok.text == "!":
            self.next()
            return f"(!{self.unary(no_struct)})"
        if tok.text == "*":
            self.next()
            inner = self.unary(no_struct)
            return inner if inner in self.refs else f"(*{inner})"
        if tok.text == "&":
            self.next()
            if self.at("mut"):
                self.next()
            return self.unary(no_struct)
        return self.postfix(self.primary(no_struct), raw_iter)

    def args(self) -> list[str]:
        self.expect("(")
        out = []
        while not self.at(")"):
            out.append(self.expr())
            if self.at(","):
                self.next()
        self.expect(")")
        return out

    def closure(self) -> str:
        self.expect("|")
        params = []
        while not self.at("|"):
            params.append(self.pattern()[0])
            if self.at(","):
                self.next()
        self.expect("|")
        body = self.expr()
        return "[&](" + ", ".join(f"auto {p}" for p in params) + f") {{ return {body}; }}"

    def postfix(self, e: str, raw_iter: bool = False):
        while True:
            tok = self.peek()
            if tok is None:
                return e
            if tok.text == "[":
                self.next()
                idx = self.expr()
                self.expect("]")
                e = f"{e}[{idx}]"
            elif tok.text == "." and self.peek(1).kind == "num":
                self.next()
                e = f"std::get<{self.next().text}>({e})"
            elif tok.text == "." and self.peek(1).kind == "id":
                self.next()
                name = self.next().text
                if not self.at("("):
                    e = f"{e}.{name}"
                    continue
                if name in ("iter", "iter_mut") and raw_iter:
                    self.args()
                    if self.at(".") and self.at("zip", 1):
                        self.next()
                        self.next()
                        (b,) = self.args()
                        return (e, b)
                    return e + ("/*iter_mut*/" if name == "iter_mut" else "/*iter*/")
                if name == "iter" and self.at(".", 2) and self.at("map", 3):
                    self.args()
                    self.next()
                    self.next()
                    self.expect("(")
                    f = self.closure()
                    self.expect(")")
                    self.expect(".")
                    red = self.next().text
                    self.args()
                    if red != "sum":
                        raise SyntaxError(f"iterator reduction {red} not translated")
                    e = f"rs::sum_map({e}, {f})"
                    continue
                args = self.args()
                if name in self.env.methods:
                    e = f"m_{name}(" + ", ".join([e, *args]) + ")"
                elif name in FLOAT_METHODS:
                    e = f"rs::{name}(" + ", ".join([e, *args]) + ")"
                elif name == "push":
                    e = f"{e}.push_back({args[0]})"
                else:
                    e = f"rs::method_{name}(" + ", ".join([e, *args]) + ")"
            elif tok.text == "(":
                args = self.args()
                e = f"{e}(" + ", ".join(args) + ")"
            else:
                return e

    def primary(self, no_struct: bool) -> str:
        tok = self.peek()
        if tok.kind == "num":
            self.next()
            return self.number(tok.text)
        if tok.kind == "str":
            self.next()
            return tok.text
        if tok.text == "(":
            self.next()
            items = []
            while not self.at(")"):
                items.append(self.expr())
                if self.at(","):
                    self.next()
                    if self.at(")"):
                        items.append(None)
            self.expect(")")
            items = [x for x in items if x is not None]
            if len(items) == 1 and not self.t[self.i - 2].text == ",":
                return f"({items[0]})"
            return "std::make_tuple(" + ", ".join(items) + ")"
        if tok.text == "[":
            self.next()
            if self.at("]"):
                self.next()
                return "rs::arr()"
            first = self.expr()
            if self.at(";"):
                self.next()
                n = self.expr()
                self.expect("]")
                return f"rs::rep<{n}>({first})"
            items = [first]
            while self.at(","):
                self.next()
                if self.at("]"):
                    break
                items.append(self.expr())
            self.expect("]")
            return "rs::arr(" + ", ".join(items) + ")"
        if tok.text == "{":
            return self.iife(lambda v: self.block_stmts(v))
        if tok.text == "if":
            return self.if_expr()
        if tok.text == "match":
            self.next()
            scrut = self.expr(no_struct=True)
            arms = self.match_arms()
            return self.iife(lambda v: self.match_code(scrut, arms, v))
        if tok.text == "|":
            return self.closure()
        if tok.kind == "id":
            path = self.path_text()
            if not no_struct and self.at("{") and (path[0].isupper()):
                return self.struct_literal(path)
            return self.resolve_path(path)
        raise SyntaxError(f"unexpected token {tok.text!r} in expression")

    def number(self, text: str) -> str:
        t = text.replace("_", "")
        m = re.match(r"^([\d.eE+-]+?)(f32|f64|u8|u16|u32|u64|usize|i8|i16|i32|i64|isize)?$", t)
        digits, suffix = m.group(1), m.group(2)
        is_float = suffix in ("f32", "f64") or "." in digits or "e" in digits or "E" in digits
        if is_float:
            if "." not in digits and "e" not in digits and "E" not in digits:
                digits += ".0"
            if digits.endswith("."):
                digits += "0"
            return digits if suffix == "f64" else digits + "f"
        if suffix:
            return f"static_cast<{PRIM[suffix]}>({digits})"
        return digits

    def resolve_path(self, path: str) -> str:
        if path in ("std::f32::consts::PI", "PI"):
            return "rs::PI_F32"
        m = re.fullmatch(r"(?:std::)?mem::size_of<(.+)>", path)
        if m:
            return f"rs::size_of<{m.group(1)}>"
        if path == "true" or path == "false":
            return path
        if "::" in path:
            owner, name = path.rsplit("::", 1)
            if owner in self.env.module_enums:
                return f"{owner}::{name}"
            if f"{owner}::{name}" in self.env.assoc:
                return f"{owner}__{name}"
            return "rs::" + path.replace("::", "_")
        return path

    def struct_literal(self, name: str) -> str:
        self.expect("{")
        var = self.fresh("s")
        stmts = [f"{name} {var}{{}};"]
        while not self.at("}"):
            fname = self.next().text
            if self.at(":"):
                self.next()
                val = self.expr()
            else:
                val = fname
            stmts.append(f"{var}.{fname} = {val};")
            if self.at(","):
                self.next()
        self.expect("}")
        stmts.append(f"return {var};")
        return "[&]() { " + " ".join(stmts) + " }()"

    def iife(self, gen) -> str:
        stmts = gen("return")
        return "[&]() { " + " ".join(stmts) + " }()"

    def if_expr(self) -> str:
        # if c { e1 } else { e2 } with single-expression branches -> ternary
        save = self.i
        self.expect("if")
        cond = self.expr(no_struct=True)
        simple = True
        branches = []
        for k in range(2):
            if not self.at("{"):
                simple = False
                break
            start = self.i
            self.next()
            depth, j = 1, self.i
            while depth:
                tx = self.t[j].text
                depth += tx == "{"
                depth -= tx == "}"
                j += 1
            inner = self.t[start + 1:j - 1]
            if any(t.text in (";", "let", "return") for t in inner):
                simple = False
                break
            sub = Body(inner, self.env, self.owner)
            sub.refs = set(self.refs)
            branches.append(sub.expr())
            self.i = j
            if k == 0:
                if not self.at("else"):
                    simple = False
                    break
                self.next()
                if self.at("if"):
                    simple = False
                    break
        if simple:
            return f"(({cond}) ? ({branches[0]}) : ({branches[1]}))"
        self.i = save
        return self.iife(lambda v: self.if_stmt(v))


class Translator:
    def __init__(self, modules: list[Module]):
        self.module_structs = {}
        self.module_enums = {}
        self.all_fns = {}
        for m in modules:
            self.module_structs.update(m.structs)
            self.module_enums.update(m.enums)
            self.all_fns.update(m.fns)
        self.methods: set[str] = set()
        self.assoc: set[str] = set()

    def cpp_struct(self, s: StructItem) -> str:
        lines = [f"struct {s.name} {{"]
        for fname, ty in s.fields:
            lines.append(f"  {ty} {fname}{{}};")
        lines.append("};")
        return "\n".join(lines)

    def cpp_enum(self, e: EnumItem) -> str:
        body = ", ".join(f"{n} = {v}" for n, v in e.variants)
        return f"enum class {e.name} : int32_t {{ {body} }};"

    def signature(self, f: FnItem) -> str:
        params = []
        if f.self_kind:
            q = "" if f.self_kind in ("mut", "val") else "const "
            amp = "" if f.self_kind == "val" else "&"
            params.append(f"{q}{f.owner} {amp}self")
        params += [f"{ty} {name}" for name, ty in f.params]
        if f.owner is None:
            fname = f"rs_{f.name}"
        elif f.self_kind:
            fname = f"m_{f.name}"
        else:
            fname = f"{f.owner}__{f.name}"
        return f"static {f.ret} {fname}(" + ", ".join(params) + ")"

    def cpp_fn(self, f: FnItem) -> str:
        body = Body([Tok("op", "{"), *f.body, Tok("op", "}")], self, f.owner)
        value = None if f.ret == "void" else "return"
        stmts = body.block_stmts(value)
        return self.signature(f) + " {\n" + indent(stmts) + "\n}"

    def translate(self, structs: list[str], enums: list[str], fns: list[str],
                  namespace: str, after_structs: str = "") -> str:
        for key in fns:
            f = self.all_fns[key]
            if f.owner and f.self_kind:
                self.methods.add(f.name)
            elif f.owner:
                self.assoc.add(key)
        # free functions are called by their Rust name; give them the rs_ prefix
        out = [f"namespace {namespace} {{"]
        out += [self.cpp_enum(self.module_enums[e]) for e in enums]
        out += [self.cpp_struct(self.module_structs[s]) for s in structs]
        if after_structs:
            out.append(after_structs)
        out += [self.signature(self.all_fns[k]) + ";" for k in fns]
        for k in fns:
            code = self.cpp_fn(self.all_fns[k])
            for free in (n for n in fns if "::" not in n):
                code = re.sub(rf"(?<![\w:.]){free}\(", f"rs_{free}(", code)
            out.append(code)
        out.append(f"}}  // namespace {namespace}")
        return "\n\n".join(out) + "\n"


def indent(stmts: list[str]) -> str:
    out, depth = [], 1
    for s in stmts:
        if s.startswith("}"):
            depth -= 1
        out.append("  " * max(depth, 0) + s)
        if s.endswith("{"):
            depth += 1
    return "\n".join(out)


def parse_file(path) -> Module:
    from pathlib import Path
    return Parser(tokenize(Path(path).read_text())).module()
