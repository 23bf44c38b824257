"""Mechanical WGSL -> C++ translation of fluid-toy's step shaders.

TEST INFRASTRUCTURE ONLY. The reference's compute path exists only as WGSL
(src/shaders/*.wgsl), which needs wgpu/naga and a GPU adapter to run; neither
exists here. This script reads those shader files where they lie and emits
C++ with the same statements, in the same order, so that the reference's own
arithmetic can run on the CPU. Its output goes only to oracle/_ref/ (never
committed) and is used to pin the hand-written oracle restatement
(oracle/sph_oracle.cpp) and to generate the committed golden fixtures.

The translation covers the WGSL subset those shaders use: structs, module
bindings, workgroup variables, constants, functions and compute entry points,
let/var declarations, if/for/switch, vector constructors, swizzles, atomics and
workgroupBarrier. The C++ meaning of every builtin is in ref_runtime.hpp.
"""
from __future__ import annotations

import re
import sys
from dataclasses import dataclass, field

TOKEN_RE = re.compile(r"""
    (?P<ws>\s+)
  | (?P<comment>//[^\n]*|/\*.*?\*/)
  | (?P<attr>@[A-Za-z_]\w*)
  | (?P<num>0[xX][0-9a-fA-F]+[iu]?|(?:\d+\.\d*|\.\d+|\d+)(?:[eE][+-]?\d+)?[fiu]?)
  | (?P<id>[A-Za-z_]\w*)
  | (?P<op>->|\+\+|--|&&|\|\||<=|>=|==|!=|<<|>>|[-+*/%&|^!~<>=]=?|[(){}\[\];:,.?])
""", re.X | re.S)


@dataclass
class Tok:
    kind: str
    text: str


def tokenize(src: str) -> list[Tok]:
    out: list[Tok] = []
    pos = 0
    while pos < len(src):
        m = TOKEN_RE.match(src, pos)
        if not m:
            raise SyntaxError(f"cannot tokenize near: {src[pos:pos + 40]!r}")
        pos = m.end()
        kind = m.lastgroup
        if kind in ("ws", "comment"):
            continue
        out.append(Tok(kind, m.group(kind)))
    return out


SWIZZLES = {"xyz", "xz", "xy", "yz"}
CONVERSIONS = {"i32", "u32", "f32"}


def fix_number(t: str) -> str:
    if t[:2] in ("0x", "0X"):
        return t[:-1] if t.endswith("i") else t
    if t.endswith("i"):
        return t[:-1]
    if t.endswith("u"):
        return t
    if t.endswith("f"):
        return t
    if "." in t or "e" in t or "E" in t:
        return t + "f"
    return t


class Translator:
    def __init__(self, toks: list[Tok], namespace: str):
        self.t = toks
        self.i = 0
        self.ns = namespace
        self.structs: list[str] = []
        self.globals: list[str] = []
        self.workgroup_vars: list[str] = []
        self.consts: list[str] = []
        self.fn_decls: list[str] = []
        self.fn_defs: list[str] = []
        self.entries: list[tuple[str, int]] = []  # (name, workgroup size)
        self.barrier_fns: set[str] = set()
        self.calls: dict[str, set[str]] = {}
        self.pending: list = []
        self.coroutines: set[str] = set()

    # -- token helpers --------------------------------------------------------
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
            raise SyntaxError(f"expected {text!r}, got {tok.text!r}")
        return tok

    def read_balanced(self, open_: str, close: str) -> list[Tok]:
        """Tokens between a matching pair; the opener is the current token."""
        self.expect(open_)
        depth = 1
        out = []
        while True:
            tok = self.next()
            if tok.text == open_:
                depth += 1
            elif tok.text == close:
                depth -= 1
                if depth == 0:
                    return out
            out.append(tok)

    def read_type(self) -> str:
        """Read a WGSL type starting at the current token; return C++ type text."""
        name = self.next().text
        if self.peek() is not None and self.peek().text == "<":
            self.next()
            args = []
            depth = 1
            cur: list[str] = []
            while depth:
                tok = self.next()
                pieces = [">", ">"] if tok.text == ">>" else [tok.text]
                for p in pieces:
                    if p == "<":
                        depth += 1
                        cur.append(p)
                    elif p == ">":
                        depth -= 1
                        if depth == 0:
                            args.append(" ".join(cur))
                            break
                        cur.append(p)
                    elif p == "," and depth == 1:
                        args.append(" ".join(cur))
                        cur = []
                    else:
                        cur.append(p)
            args = [self.type_text(a) for a in args]
            if name == "atomic":
                return args[0]
            if name == "texture_storage_3d":  # only r32float write volumes occur
                return "texture_storage_3d_r32f"
            if name == "array":
                if len(args) == 1:
                    return f"__runtime_array<{args[0]}>"
                return f"array<{args[0]}, {args[1].rstrip('u')}>"
            return f"{name}<{', '.join(args)}>"
        return name

    @staticmethod
    def type_text(s: str) -> str:
        s = s.replace(" ", "")
        s = re.sub(r"atomic<([^<>]+)>", r"\1", s)
        s = re.sub(r"<([^<>,]+),(\d+)u?>", r"<\1, \2>", s)
        return s

    # -- expressions / statements ---------------------------------------------------
    def emit_expr(self, toks: list[Tok], fn: str | None = None) -> str:
        out: list[str] = []
        n = len(toks)
        k = 0
        while k < n:
            tok = toks[k]
            txt = tok.text
            nxt = toks[k + 1].text if k + 1 < n else ""
            prev = toks[k - 1].text if k > 0 else ""
            if tok.kind == "num":
                out.append(fix_number(txt))
            elif tok.kind == "id" and txt in CONVERSIONS and nxt == "(" and prev != "<":
                out.append(f"convert<{txt}>")
            elif tok.kind == "id" and prev == "." and txt in SWIZZLES:
                out.append(txt + "()")
            elif tok.kind == "id" and nxt == "(" and fn is not None:
                self.calls.setdefault(fn, set()).add(txt)
                out.append(txt)
            else:
                out.append(txt)
            k += 1
        s = " ".join(out)
        s = re.sub(r"\s*\.\s*", ".", s)
        s = re.sub(r"(\d)\s*\.\s*(\d)", r"\1.\2", s)
        s = re.sub(r"\b(vec[234])\s*<\s*(\w+)\s*>", r"\1<\2>", s)
        s = re.sub(r",\s*\)", ")", s)  # WGSL allows a trailing comma in calls
        return s

    def translate_block(self, fn: str, body: list[Tok], indent: str = "  ") -> str:
        """Translate a function body (tokens between its braces)."""
        self._bt = body
        self._bi = 0
        return self._stmts(fn, indent, until=None)

    def _bpeek(self, k: int = 0) -> Tok | None:
        j = self._bi + k
        return self._bt[j] if j < len(self._bt) else None

    def _bnext(self) -> Tok:
        tok = self._bt[self._bi]
        self._bi += 1
        return tok

    def _until(self, stop: set[str]) -> list[Tok]:
        out = []
        depth = 0
        while True:
            tok = self._bpeek()
            if tok is None:
                return out
            if depth == 0 and tok.text in stop:
                return out
            if tok.text in "([{":
                depth += 1
            elif tok.text in ")]}":
                depth -= 1
            out.append(self._bnext())

    def _decl(self, fn: str, const: bool) -> str:
        name = self._bnext().text
        typ = None
        if self._bpeek().text == ":":
            self._bnext()
            typ = self._type_in_body()
        init = None
        if self._bpeek().text == "=":
            self._bnext()
            init = self.emit_expr(self._until({";"}), fn)
        q = "const " if const else ""
        if init is None:
            return f"{typ} {name}{{}}"
        return f"{q}{typ or 'auto'} {name} = {init}"

    def _type_in_body(self) -> str:
        saved_t, saved_i = self.t, self.i
        self.t, self.i = self._bt, self._bi
        typ = self.read_type()
        self._bi = self.i
        self.t, self.i = saved_t, saved_i
        return typ

    def _stmts(self, fn: str, indent: str, until: str | None) -> str:
        lines = []
        while True:
            tok = self._bpeek()
            if tok is None:
                break
            if until is not None and tok.text == until:
                self._bnext()
                break
            lines.append(self._stmt(fn, indent))
        return "\n".join(lines)

    def _stmt(self, fn: str, indent: str) -> str:
        tok = self._bnext()
        t = tok.text
        if t in ("let", "var"):
            if self._bpeek().text == "<":  # var<function>
                self._until({">"})
                self._bnext()
            s = self._decl(fn, const=(t == "let"))
            self._bnext()  # ;
            return f"{indent}{s};"
        if t == "if":
            cond = self._paren_or_expr(fn)
            self._expect_b("{")
            body = self._stmts(fn, indent + "  ", until="}")
            out = f"{indent}if ({cond}) {{\n{body}\n{indent}}}"
            while self._bpeek() is not None and self._bpeek().text == "else":
                self._bnext()
                if self._bpeek().text == "if":
                    self._bnext()
                    cond = self._paren_or_expr(fn)
                    self._expect_b("{")
                    body = self._stmts(fn, indent + "  ", until="}")
                    out += f" else if ({cond}) {{\n{body}\n{indent}}}"
                else:
                    self._expect_b("{")
                    body = self._stmts(fn, indent + "  ", until="}")
                    out += f" else {{\n{body}\n{indent}}}"
            return out
        if t == "for":
            self._expect_b("(")
            init_kw = self._bpeek().text
            if init_kw in ("var", "let"):
                self._bnext()
                init = self._decl(fn, const=False)
            else:
                init = self.emit_expr(self._until({";"}), fn)
            self._expect_b(";")
            cond = self.emit_expr(self._until({";"}), fn)
            self._expect_b(";")
            upd = self.emit_expr(self._until({")"}), fn)
            self._expect_b(")")
            self._expect_b("{")
            body = self._stmts(fn, indent + "  ", until="}")
            return f"{indent}for ({init}; {cond}; {upd}) {{\n{body}\n{indent}}}"
        if t == "switch":
            sel = self._paren_or_expr(fn, stop="{")
            self._expect_b("{")
            clauses = []
            while self._bpeek().text != "}":
                kw = self._bnext().text
                labels = []
                if kw == "default":
                    labels.append("default:")
                else:
                    assert kw == "case", kw
                    items = self._until({":", "{"})
                    cur = []
                    for it in items + [Tok("op", ",")]:
                        if it.text == ",":
                            if cur:
                                lab = self.emit_expr(cur, fn)
                                labels.append("default:" if lab == "default" else f"case {lab}:")
                            cur = []
                        else:
                            cur.append(it)
                if self._bpeek().text == ":":
                    self._bnext()
                self._expect_b("{")
                body = self._stmts(fn, indent + "    ", until="}")
                clauses.append(f"{indent}  {' '.join(labels)} {{\n{body}\n{indent}  }} break;")
            self._bnext()  # }
            return f"{indent}switch ({sel}) {{\n" + "\n".join(clauses) + f"\n{indent}}}"
        if t == "return":
            e = self._until({";"})
            self._bnext()
            kw = "co_return" if fn in self.coroutines else "return"
            return f"{indent}{kw} {self.emit_expr(e, fn)};".replace(f"{kw} ;", f"{kw};")
        if t in ("continue", "break"):
            self._bnext()
            return f"{indent}{t};"
        if t == "{":
            body = self._stmts(fn, indent + "  ", until="}")
            return f"{indent}{{\n{body}\n{indent}}}"
        # expression / assignment statement
        toks = [tok] + self._until({";"})
        self._bnext()
        if tok.text == "workgroupBarrier":
            return f"{indent}co_await barrier_point{{}};"
        if tok.kind == "id" and tok.text in self.coroutines:
            return f"{indent}co_await {self.emit_expr(toks, fn)};"
        return f"{indent}{self.emit_expr(toks, fn)};"

    def _expect_b(self, text: str) -> None:
        tok = self._bnext()
        if tok.text != text:
            raise SyntaxError(f"expected {text!r}, got {tok.text!r}")

    def _paren_or_expr(self, fn: str, stop: str = "{") -> str:
        toks = self._until({stop})
        s = self.emit_expr(toks, fn)
        if toks and toks[0].text == "(" and toks[-1].text == ")":
            return s[1:-1].strip() if s.startswith("(") and s.endswith(")") else s
        return s

    # -- top level -------------------------------------------------------------------
    def run(self) -> str:
        while self.peek() is not None:
            attrs = []
            while self.peek().kind == "attr":
                a = self.next().text
                args = self.read_balanced("(", ")") if self.peek() and self.peek().text == "(" else []
                attrs.append((a, [x.text for x in args]))
            kw = self.next().text
            if kw == ";":  # WGSL allows `struct S { ... };`
                continue
            if kw == "struct":
                self.top_struct()
            elif kw == "var":
                self.top_var(attrs)
            elif kw == "const":
                self.top_const()
            elif kw == "fn":
                self.top_fn(attrs)
            else:
                raise SyntaxError(f"unexpected top-level token {kw!r}")
        self.finish_functions()
        return self.render()

    def finish_functions(self) -> None:
        # call graph and direct barrier users from the raw tokens
        names = {p[0] for p in self.pending}
        for name, _sig, _pre, body, _e in self.pending:
            for k, tok in enumerate(body):
                nxt = body[k + 1].text if k + 1 < len(body) else ""
                if tok.kind == "id" and nxt == "(":
                    if tok.text == "workgroupBarrier":
                        self.barrier_fns.add(name)
                    elif tok.text in names:
                        self.calls.setdefault(name, set()).add(tok.text)
        self.coroutines = {p[0] for p in self.pending if self.uses_barrier(p[0])}
        for name, sig, pre, body, _e in self.pending:
            if name in self.coroutines:
                sig = "task " + sig.split(" ", 1)[1]
            self.fn_decls.append(f"static {sig};")
            code = self.translate_block(name, body)
            self.fn_defs.append(f"static {sig} {{\n{pre}{code}\n}}")

    def top_struct(self) -> None:
        name = self.next().text
        body = self.read_balanced("{", "}")
        fields = []
        k = 0
        while k < len(body):
            fname = body[k].text
            assert body[k + 1].text == ":"
            # collect type tokens until a top-level comma
            j = k + 2
            depth = 0
            typ_toks = []
            while j < len(body):
                tt = body[j].text
                if tt == "<":
                    depth += 1
                elif tt == ">":
                    depth -= 1
                elif tt == ">>":
                    depth -= 2
                if tt == "," and depth == 0:
                    break
                typ_toks.append(tt)
                j += 1
            typ = self.type_text("".join(typ_toks).replace(">>", ">>"))
            # WGSL host-shareable layout: vec3/vec4 align to 16 bytes, vec2 to 8
            align = "alignas(16) " if typ.startswith(("vec3<", "vec4<")) else (
                "alignas(8) " if typ.startswith("vec2<") else "")
            fields.append(f"  {align}{typ} {fname};")
            k = j + 1
        self.structs.append(f"struct {name} {{\n" + "\n".join(fields) + "\n};")

    def top_var(self, attrs) -> None:
        space = None
        if self.peek().text == "<":
            inner = self.read_balanced("<", ">")
            space = inner[0].text
        name = self.next().text
        self.expect(":")
        typ = self.read_type()
        self.expect(";")
        if space == "workgroup":
            self.globals.append(f"inline {typ} {name}{{}};")
            self.workgroup_vars.append(name)
        elif typ.startswith("__runtime_array<"):
            inner_t = typ[len("__runtime_array<"):-1]
            self.globals.append(f"inline {inner_t} *{name} = nullptr;")
        else:
            self.globals.append(f"inline {typ} {name}{{}};")

    def top_const(self) -> None:
        name = self.next().text
        typ = "auto"
        if self.peek().text == ":":
            self.next()
            typ = self.read_type()
        self.expect("=")
        toks = []
        while self.peek().text != ";":
            toks.append(self.next())
        self.next()
        self.consts.append(f"inline constexpr {typ} {name} = {self.emit_expr(toks)};")

    def top_fn(self, attrs) -> None:
        name = self.next().text
        params = self.read_balanced("(", ")")
        ret = "void"
        if self.peek().text == "->":
            self.next()
            ret = self.read_type()
        body = self.read_balanced("{", "}")
        is_entry = any(a == "@compute" for a, _ in attrs)
        # parameters
        plist = []
        builtins = []
        k = 0
        while k < len(params):
            bname = None
            if params[k].kind == "attr":
                if params[k].text == "@builtin":
                    bname = params[k + 2].text
                    k += 4
                else:
                    k += 1
                    continue
            pname = params[k].text
            assert params[k + 1].text == ":"
            saved_t, saved_i = self.t, self.i
            self.t, self.i = params, k + 2
            ptype = self.read_type()
            k = self.i
            self.t, self.i = saved_t, saved_i
            if k < len(params) and params[k].text == ",":
                k += 1
            if bname:
                builtins.append((bname, pname, ptype))
            else:
                plist.append(f"{ptype} {pname}")
        fname = f"{name}"
        if is_entry:
            wg = (1, 1, 1)
            for a, args in attrs:
                if a == "@workgroup_size":
                    dims = [int(re.sub(r"[iu]$", "", x)) for x in args if x != ","]
                    wg = tuple(dims + [1] * (3 - len(dims)))
            self.entries.append((name, wg))
            sig = f"void {fname}(uvec3 __gid, uvec3 __lid, uvec3 __wid)"
            prelude = []
            for bname, pname, ptype in builtins:
                src = {"global_invocation_id": "__gid", "local_invocation_id": "__lid",
                       "workgroup_id": "__wid"}[bname]
                prelude.append(f"  const {ptype} {pname} = {src};")
            pre = "\n".join(prelude) + ("\n" if prelude else "")
        else:
            sig = f"{ret} {fname}({', '.join(plist)})"
            pre = ""
        self.pending.append((name, sig, pre, body, is_entry))

    def uses_barrier(self, fn: str, seen=None) -> bool:
        seen = seen or set()
        if fn in self.barrier_fns:
            return True
        seen.add(fn)
        return any(self.uses_barrier(c, seen) for c in self.calls.get(fn, ()) if c not in seen)

    def render(self) -> str:
        out = [f"namespace {self.ns} {{", "using namespace wgsl;"]
        out += self.structs + self.consts + self.globals + self.fn_decls + self.fn_defs
        for name, wg3 in self.entries:
            if wg3[1] != 1 or wg3[2] != 1:
                assert name not in self.coroutines, "3-D workgroups with barriers"
                out.append(
                    f"inline void dispatch_{name}(u32 gx, u32 gy, u32 gz) {{\n"
                    f"  dispatch_sequential_3d(gx, gy, gz, uvec3({wg3[0]}u, {wg3[1]}u, {wg3[2]}u),\n"
                    f"                         [](uvec3 g, uvec3 l, uvec3 w) {{ {name}(g, l, w); }});\n}}")
                continue
            wg = wg3[0]
            if name in self.coroutines:
                resets = " ".join(f"{v} = {{}};" for v in self.workgroup_vars)
                out.append(
                    f"inline void dispatch_{name}(u32 groups) {{\n"
                    f"  dispatch_barriers(groups, {wg}u, [] {{ {resets} }},\n"
                    f"                    [](uvec3 g, uvec3 l, uvec3 w) {{ return {name}(g, l, w); }});\n}}")
            else:
                out.append(
                    f"inline void dispatch_{name}(u32 groups) {{\n"
                    f"  dispatch_sequential(groups, {wg}u,\n"
                    f"                      [](uvec3 g, uvec3 l, uvec3 w) {{ {name}(g, l, w); }});\n}}")
        out.append(f"}}  // namespace {self.ns}")
        return "\n\n".join(out)


def translate(src: str, namespace: str) -> str:
    return Translator(tokenize(src), namespace).run()


if __name__ == "__main__":
    ns = sys.argv[2] if len(sys.argv) > 2 else "shader"
    print(translate(open(sys.argv[1]).read(), ns))
