"""Source converter: C programs -> translation units for the device MPI runtime.

Replaces the clang tool `source_converter/converter.cpp` and the rewriting half
of `scripts/gpumpicc.py` with a token-level rewriter over a light C parser, so
no clang is needed.  It applies the same rules to the same C subset:

* every function written in the file gets `__device__`
  (converter.cpp:64-87); `main` becomes `__gpu_main(int argc, char** argv)`
  followed by `__gpu_max_threads()` returning the rank limit (:69-81);
* old-style (K&R) parameter lists become prototype lists (:89-122);
* a `void*` value stored into a typed pointer gets the explicit cast that C
  adds implicitly (:124-128; only the casts C++ needs are written);
* every variable with static storage (file scope, `extern`, function
  `static`) becomes `__device__ T name[MAX_RANKS]` with its initialiser
  replicated, and every use becomes `__gpu_global(name)` (:130-177, also
  inside `#define` bodies, as the clang tool rewrites spelling locations);
* identifiers spelled like C++-only keywords are renamed `__decl_<name>`
  (:178-183 renames `class`; the other C++ keywords get the same treatment);
* `#include <x>` / `"x"` become `x.cuh` (gpumpicc.py:196-201); project
  headers are converted to `x.cuh` beside the source;
* with an allocator version > 0, the coalescing arguments of
  converter.cpp:184-239/:263-318 are added.

Where the clang tool emits code that does not compile as C++ (a replicated
global declared with `[]`, `main` with differently named parameters, a `(void)`
parameter list given the coalescing flag, an empty `()` prototype of a
function defined with parameters), the converter emits the form that does.
Read-only globals (a `const` object, or an array of them) are identical in
every rank and are not replicated.
"""

from __future__ import annotations

import os
import re
import sys
from dataclasses import dataclass, field

DEFAULT_MAX_RANKS = 1024

# ---------------------------------------------------------------- lexing

_TOKEN_RE = re.compile(
    r"""
    (?P<ws>[ \t\r\f\v]+|\\\n|\n)
  | (?P<comment>/\*.*?\*/|//[^\n]*)
  | (?P<str>(?:u8|u|U|L)?"(?:\\.|[^"\\\n])*")
  | (?P<chr>(?:u|U|L)?'(?:\\.|[^'\\\n])*')
  | (?P<id>[A-Za-z_]\w*)
  | (?P<num>\.?\d(?:[eEpP][+-]|[\w.])*)
  | (?P<punct>\.\.\.|<<=|>>=|->|\+\+|--|<<|>>|<=|>=|==|!=|&&|\|\||[*/%+\-&^|]=|\#\#|[][(){}.,;:?~!<>=+\-*/%&^|\#])
    """,
    re.S | re.X,
)


@dataclass
class Tok:
    kind: str  # ws comment pp str chr id num punct
    text: str
    line: int


class ConvertError(Exception):
    pass


def _directive_end(src: str, i: int) -> int:
    """End (exclusive) of the preprocessor directive starting at src[i] == '#':
    the first newline not escaped by a backslash and not inside a block comment."""
    n = len(src)
    while i < n:
        c = src[i]
        if c == "\\" and i + 1 < n and src[i + 1] == "\n":
            i += 2
        elif c == "/" and src.startswith("/*", i):
            j = src.find("*/", i + 2)
            i = n if j < 0 else j + 2
        elif c == "/" and src.startswith("//", i):
            j = src.find("\n", i)
            return n if j < 0 else j
        elif c == '"' or c == "'":
            m = re.compile(r"%s(?:\\.|[^%s\\\n])*%s?" % (c, c, c)).match(src, i)
            i = m.end()
        elif c == "\n":
            return i
        else:
            i += 1
    return n


def lex(src: str) -> list[Tok]:
    toks: list[Tok] = []
    i, n, line = 0, len(src), 1
    at_line_start = True
    while i < n:
        if at_line_start:
            m = re.compile(r"[ \t]*#").match(src, i)
            if m:
                j = _directive_end(src, i)
                text = src[i:j]
                toks.append(Tok("pp", text, line))
                line += text.count("\n")
                i = j
                continue
        m = _TOKEN_RE.match(src, i)
        if not m:
            raise ConvertError("line %d: cannot read %r" % (line, src[i:i + 20]))
        kind = m.lastgroup
        text = m.group()
        toks.append(Tok(kind, text, line))
        nl = text.count("\n")
        line += nl
        if kind == "ws":
            if text == "\n":
                at_line_start = True
        elif kind != "comment":  # a comment leaves the "only blanks so far" state as it was
            at_line_start = False
        i = m.end()
    return toks


# ---------------------------------------------------------------- C vocabulary

STORAGE = {"typedef", "extern", "static", "auto", "register", "_Thread_local", "__thread",
           "inline", "__inline", "__inline__", "_Noreturn", "__extension__"}
QUALS = {"const", "volatile", "restrict", "__restrict", "__restrict__", "_Atomic"}
TYPE_KW = {"void", "char", "short", "int", "long", "float", "double", "signed", "unsigned",
           "_Bool", "_Complex", "complex", "bool", "__int128", "_Float128", "__signed__"}
AGGREGATE = {"struct", "union", "enum"}
CONTROL = {"if", "else", "for", "while", "do", "switch", "case", "default", "return", "goto",
           "break", "continue", "sizeof", "_Alignof", "__alignof__", "typeof", "__typeof__"}
# C identifiers that C++ reserves; `class` is the one the clang tool renames.
CXX_ONLY = {"class", "new", "delete", "this", "template", "typename", "namespace", "operator",
            "private", "protected", "public", "virtual", "friend", "explicit", "mutable", "using",
            "try", "catch", "throw", "nullptr", "export", "constexpr", "decltype", "noexcept",
            "static_assert", "thread_local", "alignas", "alignof", "char16_t", "char32_t",
            "reinterpret_cast", "static_cast", "dynamic_cast", "const_cast", "typeid", "and",
            "or", "not", "xor", "bitand", "bitor", "compl", "and_eq", "or_eq", "xor_eq", "not_eq"}

RENAME = {"restrict": "__restrict__"}


def rename(name: str) -> str:
    """C identifiers that are keywords in C++ get a prefix; C99 `restrict` is spelled as nvcc's."""
    if name in RENAME:
        return RENAME[name]
    return "__decl_" + name if name in CXX_ONLY else name


# Type names the C library and MPI headers provide.
KNOWN_TYPEDEFS = {
    "size_t", "ssize_t", "ptrdiff_t", "intptr_t", "uintptr_t", "intmax_t", "uintmax_t",
    "int8_t", "int16_t", "int32_t", "int64_t", "uint8_t", "uint16_t", "uint32_t", "uint64_t",
    "int_least8_t", "int_least16_t", "int_least32_t", "int_least64_t",
    "uint_least8_t", "uint_least16_t", "uint_least32_t", "uint_least64_t",
    "int_fast8_t", "int_fast16_t", "int_fast32_t", "int_fast64_t",
    "uint_fast8_t", "uint_fast16_t", "uint_fast32_t", "uint_fast64_t",
    "FILE", "va_list", "time_t", "clock_t", "off_t", "pid_t", "uid_t", "gid_t", "mode_t",
    "wchar_t", "div_t", "ldiv_t", "lldiv_t", "fpos_t", "DIR", "suseconds_t", "useconds_t",
    "double_t", "float_t", "sig_atomic_t", "max_align_t",
    "MPI_Comm", "MPI_Status", "MPI_Request", "MPI_Datatype", "MPI_Op", "MPI_Group", "MPI_Aint",
    "MPI_Fint", "MPI_User_function", "MPI_Errhandler", "MPI_Offset", "MPI_Info", "MPI_Win",
    "MPI_Count", "MPI_File",
}
# Library functions whose result is `void*` (the implicit conversions C++ rejects).
VOIDPTR_FUNCS = {"malloc", "calloc", "realloc", "aligned_alloc", "memcpy", "memmove", "memset",
                 "memchr", "bsearch", "__gpu_malloc", "__gpu_calloc", "__gpu_realloc"}


# ---------------------------------------------------------------- symbols


@dataclass
class VarInfo:
    ctype: str | None  # pointer type text (e.g. "INT_TYPE *") when the declarator is a simple pointer
    kind: str  # "global" (replicated, wrapped), "local", "static" (function static, wrapped), "const"


@dataclass
class FuncInfo:
    ret: str | None  # return type text when it is a simple pointer type
    params: list  # per parameter: pointer type text or None
    has_params_text: str | None = None  # definition's parameter text (for empty `()` prototypes)


@dataclass
class Symbols:
    typedefs: set = field(default_factory=lambda: set(KNOWN_TYPEDEFS))
    globals: dict = field(default_factory=dict)  # name -> VarInfo
    funcs: dict = field(default_factory=dict)  # name -> FuncInfo
    members: dict = field(default_factory=dict)  # member name -> pointer type text or "" if ambiguous
    coalesce_funcs: set = field(default_factory=set)


@dataclass
class Options:
    max_ranks: int = DEFAULT_MAX_RANKS
    malloc_version: int = 0


# ---------------------------------------------------------------- one file


class Unit:
    """One source or header file: tokens, the positions of significant tokens,
    bracket matches and the edits collected while parsing."""

    def __init__(self, src: str, path: str, syms: Symbols, opts: Options, is_header: bool):
        self.path = path
        self.syms = syms
        self.opts = opts
        self.is_header = is_header
        self.toks = lex(src)
        self.before: dict[int, list[str]] = {}
        self.after: dict[int, list[str]] = {}
        self.replace: dict[int, str] = {}
        self.sig: list[int] = []
        self._select_active()
        self.match: dict[int, int] = {}
        self._match_brackets()
        self.calls: list[tuple] = []  # (pos_callee, pos_lparen, pos_rparen, name, unconditional, func)
        self.funcdefs: list[dict] = []
        self.protos: list[dict] = []

    # ---- token access
    def t(self, p: int) -> str:
        return self.toks[self.sig[p]].text if 0 <= p < len(self.sig) else ""

    def kind(self, p: int) -> str:
        return self.toks[self.sig[p]].kind if 0 <= p < len(self.sig) else ""

    def line(self, p: int) -> int:
        return self.toks[self.sig[min(p, len(self.sig) - 1)]].line if self.sig else 0

    def ins_before(self, p: int, text: str, first: bool = False):
        lst = self.before.setdefault(self.sig[p], [])
        if first:
            lst.insert(0, text)
        else:
            lst.append(text)

    def ins_after(self, p: int, text: str):
        self.after.setdefault(self.sig[p], []).append(text)

    def repl(self, p: int, text: str):
        self.replace[self.sig[p]] = text

    def text_range(self, a: int, b: int, sub=None) -> str:
        """Source text of significant positions [a, b), with the whitespace
        between them; `sub(p)` may return replacement text for position p."""
        if a >= b:
            return ""
        out = []
        for k in range(self.sig[a], self.sig[b - 1] + 1):
            tok = self.toks[k]
            if tok.kind == "pp":
                out.append("\n" + tok.text + "\n")
                continue
            if tok.kind == "comment":
                out.append(" ")
                continue
            if sub is not None and tok.kind not in ("ws",):
                p = self._pos_of.get(k)
                if p is not None:
                    r = sub(p)
                    if r is not None:
                        out.append(r)
                        continue
            out.append(tok.text)
        return "".join(out)

    # ---- preprocessing view
    def _select_active(self):
        """Significant tokens, leaving out `#if 0` regions.  Every other
        conditional branch is kept: the parser sees all of them."""
        # region states: "on" (known taken), "off" (known not taken), "all" (unknown)
        stack = []  # per open conditional: [enclosing state, a branch known taken]
        state = "all"

        def cond(rest):
            return "off" if rest == "0" else "on" if rest == "1" else "all"

        for k, tok in enumerate(self.toks):
            if tok.kind == "pp":
                tok.inactive = state == "off"
                m = re.match(r"\s*#\s*(\w+)\s*(.*)", tok.text, re.S)
                if not m:
                    continue
                d, rest = m.group(1), m.group(2).strip()
                rest = re.sub(r"/\*.*?\*/|//.*", "", rest, flags=re.S).strip()
                if d in ("if", "ifdef", "ifndef"):
                    new = cond(rest) if d == "if" else "all"
                    stack.append([state, new == "on"])
                    state = "off" if state == "off" else new
                elif d in ("elif", "else") and stack:
                    parent, taken = stack[-1]
                    if parent == "off" or taken:
                        state = "off"
                    elif d == "else":
                        state = "on" if state == "off" else "all"
                    else:
                        state = cond(rest) if state == "off" else ("off" if cond(rest) == "off" else "all")
                    stack[-1][1] = taken or state == "on"
                elif d == "endif" and stack:
                    state = stack.pop()[0]
                continue
            if state == "off":
                tok.inactive = True
                continue
            if tok.kind in ("ws", "comment"):
                continue
            self.sig.append(k)
        self._pos_of = {k: p for p, k in enumerate(self.sig)}

    def _match_brackets(self):
        stack = []
        pairs = {")": "(", "]": "[", "}": "{"}
        for p in range(len(self.sig)):
            s = self.t(p)
            if s in ("(", "[", "{"):
                stack.append(p)
            elif s in pairs:
                if not stack or self.t(stack[-1]) != pairs[s]:
                    raise ConvertError("%s:%d: unbalanced '%s'" % (self.path, self.line(p), s))
                q = stack.pop()
                self.match[q] = p
                self.match[p] = q
        if stack:
            raise ConvertError("%s:%d: unclosed '%s'" % (self.path, self.line(stack[-1]), self.t(stack[-1])))

    def render(self) -> str:
        out = []
        for k, tok in enumerate(self.toks):
            out.extend(self.before.get(k, ()))
            if tok.kind == "pp" and k not in self.replace:
                out.append(self._rewrite_directive(tok))
            else:
                out.append(self.replace.get(k, tok.text))
            out.extend(self.after.get(k, ()))
        return "".join(out)

    # ---- directives
    def _rewrite_directive(self, tok: Tok) -> str:
        text = tok.text
        m = re.match(r'(\s*#\s*include\s*)([<"])([^>"]*)([>"])(.*)$', text, re.S)
        if m:
            name = m.group(3)
            if not name.endswith(".cuh"):
                name += ".cuh"
            return m.group(1) + m.group(2) + name + m.group(4) + m.group(5)
        if getattr(tok, "inactive", False):
            return text
        m = re.match(r"(\s*#\s*define\s+)(\w+)(\([^)]*\))?(.*)$", text, re.S)
        if not m:
            return text
        params = set()
        if m.group(3):
            params = {x.strip() for x in m.group(3)[1:-1].split(",")}
        body = m.group(4)
        return m.group(1) + m.group(2) + (m.group(3) or "") + self._wrap_text(body, params)

    def _wrap_text(self, body: str, skip: set) -> str:
        out = []
        prev = ""
        for tok in lex_fragment(body):
            s = tok.text
            if (tok.kind == "id" and s in self.syms.globals and s not in skip
                    and self.syms.globals[s].kind == "global" and prev not in (".", "->", "#", "##")):
                out.append("__gpu_global(%s)" % rename(s))
            elif tok.kind == "id":
                out.append(rename(s))
            else:
                out.append(s)
            if tok.kind not in ("ws", "comment"):
                prev = s
        return "".join(out)

    # ---- parsing entry
    def convert(self):
        p, n = 0, len(self.sig)
        while p < n:
            p = self._external(p)
        if self.sig:
            self._rename_cxx_keywords()

    def _rename_cxx_keywords(self):
        for p in range(len(self.sig)):
            if self.kind(p) == "id" and rename(self.t(p)) != self.t(p) and self.sig[p] not in self.replace:
                self.repl(p, rename(self.t(p)))

    # ---- top level
    def _external(self, p: int) -> int:
        s = self.t(p)
        if s == ";":
            return p + 1
        if s == "}":  # end of an extern "C" block
            return p + 1
        if s == "extern" and self.kind(p + 1) == "str" and self.t(p + 2) == "{":
            return p + 3
        q, in_init = p, False
        n = len(self.sig)
        while q < n:
            s = self.t(q)
            if s in ("(", "["):
                q = self.match[q] + 1
                continue
            if s == "{":
                prev, prev2 = self.t(q - 1), self.t(q - 2)
                if in_init or prev in AGGREGATE or (prev2 in AGGREGATE and self.kind(q - 1) == "id"):
                    q = self.match[q] + 1
                    continue
                end = self.match[q]
                self._function(p, q, end)
                return end + 1
            if s == "=":
                in_init = True
            elif s == ",":
                in_init = False
            elif s == ";":
                lb = self._knr_body(p, q)
                if lb is not None:
                    self._function(p, lb, self.match[lb])
                    return self.match[lb] + 1
                self._declaration(p, q, scope=None)
                return q + 1
            q += 1
        raise ConvertError("%s:%d: declaration not terminated" % (self.path, self.line(p)))

    def _knr_body(self, p: int, semi: int):
        """When p..semi is the head of an old-style definition (`f(a, b) int a;
        ...`), the position of its body's '{', else None."""
        r, info = self._specs(p, semi)
        if info is None:
            r = p
        dec = self._declarator(r, semi)
        if dec["func"] is None or dec["end"] >= semi:
            return None
        a, b = dec["func"]
        items = self._split_commas(a + 1, b)
        if not items or any(pb != pa + 1 or self.kind(pa) != "id" or self.t(pa) in self.syms.typedefs
                            or self.t(pa) in TYPE_KW for pa, pb in items):
            return None
        q = dec["end"]
        while q < len(self.sig) and self.t(q) != "{":
            q = self.match[q] + 1 if self.t(q) in ("(", "[") else q + 1
        return q if q < len(self.sig) else None

    # ---- declaration specifiers
    def _specs(self, p: int, end: int):
        """Parse declaration specifiers at p.  Returns (q, info) with q the first
        declarator position and info a dict, or (p, None) when p does not
        start a declaration."""
        info = {"storage": set(), "const": False, "has_type": False, "type_from": None,
                "type_to": None, "aggregates": []}
        q = p
        while q < end:
            s = self.t(q)
            if s in STORAGE:
                info["storage"].add(s)
                q += 1
            elif s in QUALS:
                info["const"] = True if s == "const" else info["const"]
                info["type_from"] = q if info["type_from"] is None else info["type_from"]
                info["type_to"] = q + 1
                q += 1
            elif s in ("__attribute__", "__declspec", "__align__", "__builtin_align__"):
                q = self.match[q + 1] + 1 if self.t(q + 1) == "(" else q + 1
            elif s in TYPE_KW:
                info["has_type"] = True
                info["type_from"] = q if info["type_from"] is None else info["type_from"]
                q += 1
                info["type_to"] = q
            elif s in AGGREGATE:
                info["has_type"] = True
                info["type_from"] = q if info["type_from"] is None else info["type_from"]
                q += 1
                while self.t(q) in ("__attribute__",):
                    q = self.match[q + 1] + 1
                if self.kind(q) == "id":
                    q += 1
                if self.t(q) == "{":
                    info["aggregates"].append((s, q, self.match[q]))
                    q = self.match[q] + 1
                info["type_to"] = q
            elif s in ("typeof", "__typeof__") and self.t(q + 1) == "(":
                info["has_type"] = True
                info["type_from"] = q if info["type_from"] is None else info["type_from"]
                q = self.match[q + 1] + 1
                info["type_to"] = q
            elif self.kind(q) == "id" and not info["has_type"] and s in self.syms.typedefs:
                nxt = self.t(q + 1)
                # `T x`, `T *x`, `T (x)`, `T;` — not `T = ...`, `T(...)` call, `T.x`
                if nxt in ("=", ".", "->", "[", "++", "--", "+=", "-=", ",", ")", ":", "?"):
                    break
                info["has_type"] = True
                info["type_from"] = q if info["type_from"] is None else info["type_from"]
                q += 1
                info["type_to"] = q
            else:
                break
        if q == p or not (info["has_type"] or info["storage"]):
            return p, None
        return q, info

    def type_text(self, info) -> str:
        if info["type_from"] is None:
            return "int"
        return re.sub(r"\s+", " ", self.text_range(info["type_from"], info["type_to"])).strip()

    # ---- declarators
    def _declarator(self, d: int, end: int):
        """Parse one declarator at d.  Returns dict with name (position or None),
        stars, ptr_const, func (params range), array, nested, end position."""
        res = {"name": None, "stars": 0, "ptr_const": False, "func": None, "array": False,
               "nested": False, "dims": [], "start": d}
        while d < end and (self.t(d) == "*" or self.t(d) in QUALS or self.t(d) == "__attribute__"):
            if self.t(d) == "*":
                res["stars"] += 1
                res["ptr_const"] = False
            elif self.t(d) == "const" and res["stars"]:
                res["ptr_const"] = True
            if self.t(d) == "__attribute__":
                d = self.match[d + 1] + 1
            else:
                d += 1
        if self.t(d) == "(" and d < end:
            inner = self._declarator(d + 1, self.match[d])
            res["name"] = inner["name"]
            res["nested"] = True
            res["inner"] = inner
            d = self.match[d] + 1
        elif self.kind(d) == "id" and self.t(d) not in STORAGE and d < end:
            res["name"] = d
            d += 1
        while d < end and self.t(d) in ("(", "["):
            if self.t(d) == "(" and res["func"] is None and not res["nested"] and res["name"] == d - 1:
                res["func"] = (d, self.match[d])
            elif self.t(d) == "[":
                res["array"] = True
                res["dims"].append((d, self.match[d]))
            elif self.t(d) == "(":
                res["fnptr"] = True
            d = self.match[d] + 1
        while d < end and (self.t(d) in ("__attribute__", "__asm__", "asm")):
            d = self.match[d + 1] + 1
        res["end"] = d
        return res

    def _init_end(self, d: int, end: int) -> int:
        while d < end and self.t(d) not in (",", ";"):
            if self.t(d) in ("(", "[", "{"):
                d = self.match[d] + 1
            else:
                d += 1
        return d

    def _declarators(self, q: int, end: int):
        """All init-declarators from q to end (the ';').  Each dict gains
        init (a, b) or None."""
        out = []
        while q < end:
            dec = self._declarator(q, end)
            q = dec["end"]
            dec["init"] = None
            if self.t(q) == "=":
                e = self._init_end(q + 1, end)
                dec["init"] = (q + 1, e)
                q = e
            out.append(dec)
            if self.t(q) == ",":
                q += 1
            elif q < end:
                # something the parser does not understand (e.g. a bit-field); stop here
                break
        return out

    def _ptr_type(self, info, dec) -> str | None:
        """Type text of a simple (non-array, non-function) pointer declarator."""
        if dec["stars"] == 0 or dec["array"] or dec["func"] or dec["nested"] or dec.get("fnptr"):
            return None
        return self.type_text(info) + " " + "*" * dec["stars"]

    def _readonly(self, info, dec) -> bool:
        if dec["nested"] or dec.get("fnptr"):
            return False
        if dec["stars"] == 0:
            return info["const"]
        return dec["ptr_const"]

    # ---- declarations
    def _declaration(self, p: int, end: int, scope):
        """Declaration from p to the ';' at end.  scope is None at file scope,
        else the innermost block scope (a dict) of a function body."""
        q, info = self._specs(p, end)
        if info is None:
            if scope is None:
                # e.g. an implicit-int declaration or a macro invocation: leave it
                return
            return
        for kind, a, b in info["aggregates"]:
            self._aggregate(kind, a, b)
        if "typedef" in info["storage"]:
            for dec in self._declarators(q, end):
                if dec["name"] is not None:
                    self.syms.typedefs.add(self.t(dec["name"]))
            return
        decs = self._declarators(q, end)
        if scope is None:
            self._file_scope_decl(p, info, decs)
        else:
            self._block_decl(p, info, decs, scope)

    def _aggregate(self, kind: str, a: int, b: int):
        if kind == "enum":
            return
        q = a + 1
        while q < b:
            e = q
            while e < b and self.t(e) != ";":
                e = self.match[e] + 1 if self.t(e) in ("(", "[", "{") else e + 1
            r, info = self._specs(q, e)
            if info is not None:
                for kk, aa, bb in info["aggregates"]:
                    self._aggregate(kk, aa, bb)
                for dec in self._declarators(r, e):
                    if dec["name"] is not None:
                        name = self.t(dec["name"])
                        ty = self._ptr_type(info, dec) or ""
                        old = self.syms.members.get(name)
                        self.syms.members[name] = ty if old is None or old == ty else ""
            q = e + 1

    def _file_scope_decl(self, p: int, info, decs):
        dev = False
        for dec in decs:
            if dec["name"] is None:
                continue
            name = self.t(dec["name"])
            if dec["func"] is not None:
                self._record_func(info, dec, definition=False)
                self.protos.append({"name": name, "dec": dec, "start": p})
                dev = True
                continue
            dev = True
            if self._readonly(info, dec):
                self.syms.globals.pop(name, None)
                continue
            self.syms.globals[name] = VarInfo(self._ptr_type(info, dec), "global")
            self._replicate(dec)
        if dev:
            self.ins_before(p, "__device__ ")

    def _replicate(self, dec, lookup=None):
        """`name` -> `name[MAX]`, initialiser replicated once per rank slot.  A
        reference to another replicated variable in the initialiser (an address
        or an array that decays) takes that variable's element of the same slot."""
        R = self.opts.max_ranks
        name = dec["name"]
        dims = dec["dims"]
        lookup = lookup or self.syms.globals.get
        if dims and dims[0][1] == dims[0][0] + 1:
            # `T a[] = init`: the clang tool would emit `a[MAX][]`; give the size
            if dec["init"] is None:
                raise ConvertError("%s:%d: replicated array without size or initialiser"
                                   % (self.path, self.line(name)))
            self.ins_after(dims[0][0], self._init_count(dec["init"]))
        self.ins_after(name, "[%d]" % R)
        if dec["init"] is None:
            return
        a, b = dec["init"]
        own = self.t(name)

        def replicated(pp):
            v = lookup(self.t(pp)) if self.kind(pp) == "id" else None
            return (v is not None and v.kind in ("global", "static") and self.t(pp) != own
                    and self.t(pp - 1) not in (".", "->"))

        def per_slot(k):
            def sub(pp):
                if replicated(pp):
                    return "%s[%d]" % (rename(self.t(pp)), k)
                if self.kind(pp) == "id" and rename(self.t(pp)) != self.t(pp):
                    return rename(self.t(pp))
                return None
            return self.text_range(a, b, sub).strip()

        if any(replicated(pp) for pp in range(a, b)):
            items = [per_slot(k) for k in range(R)]
        else:
            items = [per_slot(0)] * R
        rows = [", ".join(items[i:i + 16]) for i in range(0, R, 16)]
        self.repl(a, "{" + ",\n    ".join(rows) + "}")
        for pp in range(a + 1, b):
            self.repl(pp, "")
        self._blank_between(a, b)

    def _blank_between(self, a: int, b: int):
        """Drop the blanks, comments and directives between significant positions a and b-1."""
        for k in range(self.sig[a] + 1, self.sig[b - 1] + 1):
            if self.toks[k].kind in ("ws", "comment", "pp"):
                self.replace[k] = ""

    def _init_count(self, init) -> str:
        """Element count of the initialiser of an unsized array."""
        a, b = init
        if self.t(a) != "{":
            # a string literal (or several, concatenated) for a char array
            return "sizeof(%s)" % self.text_range(a, b).strip()
        e = self.match[a]
        if e == a + 1:
            return "0"
        n, q, item_start = 1, a + 1, True
        while q < e:
            s = self.t(q)
            if item_start and s in ("[", "."):
                raise ConvertError("%s:%d: designated initialiser of an unsized replicated array"
                                   % (self.path, self.line(q)))
            item_start = False
            if s in ("(", "[", "{"):
                q = self.match[q] + 1
                continue
            if s == ",":
                item_start = True
                if q + 1 < e:
                    n += 1
            q += 1
        return str(n)

    def _record_func(self, info, dec, definition: bool):
        name = self.t(dec["name"])
        params = []
        a, b = dec["func"]
        for pa, pb in self._split_commas(a + 1, b):
            r, pinfo = self._specs(pa, pb)
            if pinfo is None:
                params.append(None)
                continue
            pdec = self._declarator(r, pb)
            params.append(self._ptr_type(pinfo, pdec) if not pdec["array"] else None)
        ret = None
        if dec["stars"] and not dec["nested"]:
            ret = self.type_text(info) + " " + "*" * dec["stars"]
        old = self.syms.funcs.get(name)
        fi = FuncInfo(ret, params)
        if old is not None and old.has_params_text is not None:
            fi.has_params_text = old.has_params_text
        if definition and b > a + 1 and not (b == a + 2 and self.t(a + 1) == "void"):
            fi.has_params_text = self.text_range(a + 1, b)
        if old is not None and len(old.params) > len(params):
            fi.params = old.params
        self.syms.funcs[name] = fi

    def _split_commas(self, a: int, b: int):
        out, q, start = [], a, a
        while q < b:
            s = self.t(q)
            if s in ("(", "[", "{"):
                q = self.match[q] + 1
                continue
            if s == ",":
                out.append((start, q))
                start = q + 1
            q += 1
        if start < b:
            out.append((start, b))
        return out

    # ---- function definitions
    def _function(self, p: int, lb: int, rb: int):
        q, info = self._specs(p, lb)
        if info is None:
            # implicit int return type (K&R) e.g. `main() { }`
            info = {"storage": set(), "const": False, "has_type": False, "type_from": None,
                    "type_to": None, "aggregates": []}
            q = p
        dec = self._declarator(q, lb)
        if dec["name"] is None or dec["func"] is None:
            raise ConvertError("%s:%d: cannot read function definition" % (self.path, self.line(p)))
        name = self.t(dec["name"])
        a, b = dec["func"]
        scope = {}
        kr_end = dec["end"]
        knr_text = None
        # K&R parameter declarations between ')' and '{'
        if kr_end < lb:
            knr_text = self._knr(dec, kr_end, lb, scope)
        else:
            for pa, pb in self._split_commas(a + 1, b):
                r, pinfo = self._specs(pa, pb)
                if pinfo is None:
                    continue
                pdec = self._declarator(r, pb)
                if pdec["name"] is not None:
                    scope[self.t(pdec["name"])] = VarInfo(self._ptr_type(pinfo, pdec), "local")
        self._record_func(info, dec, definition=True)
        if knr_text is not None:
            self.syms.funcs[name].has_params_text = knr_text
        if not info["has_type"] and info["type_from"] is None and "main" != name:
            self.ins_before(q, "int ")
        self.ins_before(p, "__device__ ", first=True)
        fdef = {"name": name, "dec": dec, "start": p, "lb": lb, "rb": rb,
                "ret": self.syms.funcs[name].ret, "allocs": False}
        self.funcdefs.append(fdef)
        if name == "main":
            self.repl(dec["name"], "__gpu_main")
            names = [v for v in scope]
            if len(names) >= 2:
                params = "(int %s, char** %s)" % (names[0], names[1])
            else:
                params = "(int argc, char** argv)"
                scope = {"argc": VarInfo(None, "local"), "argv": VarInfo(None, "local")}
            self.repl(a, params)
            for pp in range(a + 1, b + 1):
                self.repl(pp, "")
            self._blank_between(a, b + 1)
            if not info["has_type"]:
                self.ins_before(dec["name"], "int ")
            self.ins_after(rb, "\n\n__device__ int __gpu_max_threads() {\n    return %d;\n}\n" % self.opts.max_ranks)
        self._body(lb, rb, [scope], fdef)

    def _knr(self, dec, a0: int, lb: int, scope):
        a, b = dec["func"]
        names = [self.t(pa) for pa, pb in self._split_commas(a + 1, b) if pb == pa + 1 and self.kind(pa) == "id"]
        decls = {}
        q = a0
        while q < lb:
            e = q
            while e < lb and self.t(e) != ";":
                e = self.match[e] + 1 if self.t(e) in ("(", "[") else e + 1
            r, info = self._specs(q, e)
            if info is None:
                raise ConvertError("%s:%d: cannot read K&R parameter declaration" % (self.path, self.line(q)))
            ty = self.type_text(info)
            for pdec in self._declarators(r, e):
                if pdec["name"] is None:
                    continue
                nm = self.t(pdec["name"])
                decls[nm] = (ty + " " + self.text_range(pdec["start"], pdec["end"]).strip(),
                             self._ptr_type(info, pdec))
            q = e + 1
        parts = []
        for nm in names:
            text, ptr = decls.get(nm, ("int " + nm, None))
            parts.append(text)
            scope[nm] = VarInfo(ptr, "local")
        self.repl(a, "(" + ", ".join(parts) + ")")
        for pp in range(a + 1, b + 1):
            self.repl(pp, "")
        for pp in range(a0, lb):
            self.repl(pp, "")
        self._blank_between(a, lb)
        return ", ".join(parts)

    # ---- statements
    def _stmt_end(self, p: int) -> int:
        """Position just after the statement starting at p."""
        s = self.t(p)
        if s == "{":
            return self.match[p] + 1
        if s == "if":
            e = self._stmt_end(self.match[p + 1] + 1)
            if self.t(e) == "else":
                e = self._stmt_end(e + 1)
            return e
        if s in ("for", "while", "switch"):
            return self._stmt_end(self.match[p + 1] + 1)
        if s == "do":
            e = self._stmt_end(p + 1)
            # while ( ... ) ;
            return self.match[e + 1] + 2
        if self.kind(p) == "id" and self.t(p + 1) == ":" and s not in ("default",):
            return self._stmt_end(p + 2)
        if s == "case" or s == "default":
            q = p
            while self.t(q) != ":":
                q = self.match[q] + 1 if self.t(q) in ("(", "[") else q + 1
            return self._stmt_end(q + 1)
        q = p
        n = len(self.sig)
        while q < n and self.t(q) != ";":
            if self.t(q) in ("(", "[", "{"):
                q = self.match[q] + 1
            else:
                q += 1
        return q + 1

    def _lookup(self, scopes, name):
        for sc in reversed(scopes):
            if name in sc:
                return sc[name]
        return self.syms.globals.get(name)

    def _body(self, lb: int, rb: int, scopes, fdef):
        """Walk a function body: block scopes, declarations, references to
        globals, casts, and the call sites the coalescing rules need."""
        cond_until = []  # end positions of enclosing if/for/while/do statements
        pops = {}  # position -> scopes to pop when reaching it
        scopes = scopes + [{}]
        q = lb + 1
        stmt_start = True
        stmt_first = lb + 1  # first position of the current statement
        while q < rb:
            while pops.get(q):
                pops[q] -= 1
                scopes.pop()
            cond_until = [e for e in cond_until if e > q]
            s = self.t(q)
            if stmt_start:
                stmt_first = q
                # declaration?
                if self.kind(q) == "id" and self.t(q + 1) != ":" or s in STORAGE or s in AGGREGATE:
                    r, info = self._specs(q, rb)
                    if info is not None and self.t(r) != "(" or (info is not None and self._looks_decl(r)):
                        e = q
                        while self.t(e) != ";":
                            e = self.match[e] + 1 if self.t(e) in ("(", "[", "{") else e + 1
                        self._declaration_in_body(q, e, scopes, fdef, bool(cond_until))
                        q = e + 1
                        stmt_start = True
                        continue
            stmt_start = False
            if s == "{":
                scopes.append({})
                stmt_start = True
                q += 1
                continue
            if s == "}":
                scopes.pop()
                stmt_start = True
                q += 1
                continue
            if s == ";":
                stmt_start = True
                q += 1
                continue
            if s in ("if", "for", "while", "do", "switch"):
                end = self._stmt_end(q)
                if s != "switch":
                    cond_until.append(end)
                if s == "for":
                    # declarations in the for-init live until the end of the statement
                    scopes.append({})
                    pops[end] = pops.get(end, 0) + 1
                    lp = q + 1
                    r, info = self._specs(lp + 1, self.match[lp])
                    if info is not None:
                        e = lp + 1
                        while self.t(e) != ";":
                            e = self.match[e] + 1 if self.t(e) in ("(", "[", "{") else e + 1
                        self._declaration_in_body(lp + 1, e, scopes, fdef, True)
                        q = e + 1
                        continue
                    q = lp + 1
                    continue
                if s == "do":
                    stmt_start = True
                q += 1
                continue
            if s == "else":
                stmt_start = True
                q += 1
                continue
            if s == ")" and self.t(self.match[q] - 1) in ("if", "while", "switch", "for"):
                # a new statement follows the head (for: the scope was opened above)
                stmt_start = True
                q += 1
                continue
            if s in ("case", "default"):
                while self.t(q) != ":":
                    q = self.match[q] + 1 if self.t(q) in ("(", "[") else q + 1
                stmt_start = True
                q += 1
                continue
            if s == ":" and self.kind(q - 1) == "id" and self.t(q - 2) in (";", "{", "}"):
                stmt_start = True  # after a label
                q += 1
                continue
            if s == "return":
                e = self._expr_end(q + 1, rb)
                if (fdef["ret"] and not fdef["ret"].replace(" ", "").endswith("void*")
                        and self._is_voidptr(q + 1, e, scopes)):
                    self.ins_before(q + 1, "(%s)" % fdef["ret"], first=True)
                q += 1
                continue
            if s == "=" :
                self._assign_cast(q, rb, scopes)
            if self.kind(q) == "id":
                first = stmt_first
                self._ident(q, scopes, fdef, lambda: bool(cond_until) or self._in_ternary(first, rb))
            q += 1

    def _looks_decl(self, r: int) -> bool:
        # `T (*fp)(...)`-style declarator after specifiers
        return self.t(r) == "(" and self.t(r + 1) == "*"

    def _expr_end(self, q: int, rb: int) -> int:
        while q < rb and self.t(q) not in (";", ","):
            if self.t(q) in ("(", "[", "{"):
                q = self.match[q] + 1
            else:
                q += 1
        return q

    def _in_ternary(self, first: int, rb: int) -> bool:
        e = self._stmt_scan_end(first, rb)
        for k in range(first, e):
            if self.t(k) == "?":
                return True
        return False

    def _stmt_scan_end(self, q: int, rb: int) -> int:
        while q < rb and self.t(q) not in (";", "{", "}"):
            q = self.match[q] + 1 if self.t(q) in ("(", "[") else q + 1
        return q

    def _declaration_in_body(self, p: int, e: int, scopes, fdef, conditional: bool):
        q, info = self._specs(p, e)
        for kind, a, b in info["aggregates"]:
            self._aggregate(kind, a, b)
        if "typedef" in info["storage"]:
            for dec in self._declarators(q, e):
                if dec["name"] is not None:
                    self.syms.typedefs.add(self.t(dec["name"]))
            return
        decs = self._declarators(q, e)
        static = "static" in info["storage"]
        extern = "extern" in info["storage"]
        dev = False
        for dec in decs:
            if dec["name"] is None:
                continue
            name = self.t(dec["name"])
            # the declarator's own array sizes and initialiser are walked for references
            for a, b in dec["dims"]:
                self._walk_expr(a + 1, b, scopes, fdef, conditional)
            if dec["func"] is not None:
                self._record_func(info, dec, definition=False)
                dev = True
                continue
            if extern:
                continue  # refers to the global of that name
            if static and not self._readonly(info, dec):
                scopes[-1][name] = VarInfo(self._ptr_type(info, dec), "static")
                dev = True
                self._replicate_static(dec, scopes, fdef)
                continue
            if static:
                dev = True
            scopes[-1][name] = VarInfo(self._ptr_type(info, dec), "local")
            if dec["init"] is not None:
                a, b = dec["init"]
                ty = self._ptr_type(info, dec)
                if ty and not ty.replace(" ", "").startswith("void*") and self._is_voidptr(a, b, scopes):
                    self.ins_before(a, "(%s)" % ty, first=True)
                self._walk_expr(a, b, scopes, fdef, conditional)
        if dev:
            self.ins_before(p, "__device__ ")

    def _replicate_static(self, dec, scopes, fdef):
        # a function static: same form as a file-scope global; its initialiser is a constant
        self._replicate(dec, lambda nm: self._lookup(scopes, nm))

    def _walk_expr(self, a: int, b: int, scopes, fdef, conditional: bool):
        q = a
        while q < b:
            if self.t(q) == "=":
                self._assign_cast(q, b, scopes)
            if self.kind(q) == "id":
                self._ident(q, scopes, fdef, lambda: conditional or any(self.t(k) == "?" for k in range(a, b)))
            q += 1

    def _ident(self, q: int, scopes, fdef, conditional: bool):
        s = self.t(q)
        prev = self.t(q - 1)
        if prev in (".", "->", "goto") or prev in AGGREGATE:
            return
        if self.t(q + 1) == ":" and prev in (";", "{", "}"):
            return  # a label
        if self.t(q + 1) == "(":
            self._call(q, scopes, fdef, conditional)
            return
        v = self._lookup(scopes, s)
        if v is not None and v.kind in ("global", "static"):
            self.ins_before(q, "__gpu_global(")
            self.ins_after(q, ")")

    def _call(self, q: int, scopes, fdef, conditional: bool):
        name = self.t(q)
        if self._lookup(scopes, name) is not None and self._lookup(scopes, name).kind in ("global", "static"):
            # call through a replicated function pointer
            self.ins_before(q, "__gpu_global(")
            self.ins_after(q, ")")
            return
        lp = q + 1
        rp = self.match[lp]
        if self.opts.malloc_version > 0:
            self.calls.append((q, lp, rp, name, not conditional(), fdef))
        fi = self.syms.funcs.get(name)
        if fi is None:
            return
        for idx, (a, b) in enumerate(self._split_commas(lp + 1, rp)):
            if idx < len(fi.params) and fi.params[idx] and not fi.params[idx].replace(" ", "").startswith("void*"):
                if self._is_voidptr(a, b, scopes):
                    self.ins_before(a, "(%s)" % fi.params[idx], first=True)

    def _assign_cast(self, q: int, end: int, scopes):
        """`lhs = <void* expression>` where lhs has a known typed-pointer type."""
        ty = None
        p = q - 1
        if self.t(p) == "]" and self.kind(self.match[p] - 1) == "id" and self.t(self.match[p] - 2) not in (".", "->"):
            v = self._lookup(scopes, self.t(self.match[p] - 1))
            if v is not None and v.ctype and v.ctype.count("*") >= 2:
                ty = v.ctype[:v.ctype.rindex("*")].rstrip()  # "T **" -> "T *"
        elif self.kind(p) == "id":
            if self.t(p - 1) in (".", "->"):
                ty = self.syms.members.get(self.t(p)) or None
            else:
                v = self._lookup(scopes, self.t(p))
                ty = v.ctype if v is not None else None
        if not ty or ty.replace(" ", "").startswith("void*"):
            return
        e = self._expr_end(q + 1, end)
        if self._is_voidptr(q + 1, e, scopes):
            self.ins_before(q + 1, "(%s)" % ty, first=True)

    def _is_voidptr(self, a: int, b: int, scopes) -> bool:
        while b - a >= 2 and self.t(a) == "(" and self.match[a] == b - 1:
            a, b = a + 1, b - 1
        if a >= b:
            return False
        if self.kind(a) == "id" and self.t(a + 1) == "(" and self.match[a + 1] == b - 1:
            name = self.t(a)
            if name in VOIDPTR_FUNCS:
                return True
            fi = self.syms.funcs.get(name)
            return fi is not None and fi.ret is not None and fi.ret.replace(" ", "") in ("void*", "constvoid*")
        if b == a + 1 and self.kind(a) == "id":
            v = self._lookup(scopes, self.t(a))
            return v is not None and v.ctype is not None and v.ctype.replace(" ", "") == "void*"
        if b - a >= 3 and self.t(b - 2) in ("->", ".") and self.kind(b - 1) == "id":
            # a member access chain (`p->next->data`, `s.buf`) ending in a `void *` member
            q = a
            while q < b - 2:
                if self.t(q) in ("(", "["):
                    q = self.match[q] + 1
                elif self.kind(q) == "id" or self.t(q) in ("->", "."):
                    q += 1
                else:
                    return False
            return (self.syms.members.get(self.t(b - 1)) or "").replace(" ", "") == "void*"
        return False

    # ---- post-pass: coalescing arguments and empty prototypes
    def finish(self):
        if self.opts.malloc_version > 0:
            self._coalesce()
        for pr in self.protos:
            dec = pr["dec"]
            a, b = dec["func"]
            fi = self.syms.funcs.get(pr["name"])
            if b == a + 1 and fi is not None and fi.has_params_text:
                self.ins_after(a, fi.has_params_text.strip())

    def _coalesce(self):
        allocs = {"malloc", "MPI_Alltoall"}
        for fd in self.funcdefs:
            if fd["name"] == "main":
                continue
            if any(c[5] is fd and c[3] in allocs and c[4] for c in self.calls):
                self.syms.coalesce_funcs.add(fd["name"])
        for fd in self.funcdefs:
            if fd["name"] in self.syms.coalesce_funcs:
                a, b = fd["dec"]["func"]
                proto_before = any(pr["name"] == fd["name"] and pr["start"] < fd["start"] for pr in self.protos)
                self._add_param(a, b, "bool __coalesced" + ("" if proto_before else " = false"))
        for pr in self.protos:
            if pr["name"] in self.syms.coalesce_funcs:
                a, b = pr["dec"]["func"]
                self._add_param(a, b, "bool __coalesced = false")
        for q, lp, rp, name, uncond, fd in self.calls:
            if not uncond or fd is None:
                continue
            if name in allocs or name in self.syms.coalesce_funcs:
                if fd["name"] == "main":
                    arg = "true"
                elif fd["name"] in self.syms.coalesce_funcs:
                    arg = "__coalesced"
                else:
                    arg = "false"  # a caller without the flag (the clang tool emits an undeclared name)
                self.ins_before(rp, ("" if rp == lp + 1 else ", ") + arg)
                if name == "MPI_Alltoall":
                    self.repl(q, "MPI_Alltoall_coalesce")
        if self.opts.malloc_version in (3, 7):
            for fd in self.funcdefs:
                if fd["name"] != "main":
                    continue
                lb, rb = fd["lb"], fd["rb"]
                self.ins_after(lb, "\n    __gpu_init_malloc();")
                last = self._last_stmt(lb, rb)
                if last is not None:
                    self.ins_before(last, "__gpu_clean_malloc();\n    ", first=True)

    def _add_param(self, a: int, b: int, text: str):
        if b == a + 1:
            self.ins_after(a, text)
        elif b == a + 2 and self.t(a + 1) == "void":
            self.repl(a + 1, text)
        else:
            self.ins_before(b, ", " + text)

    def _last_stmt(self, lb: int, rb: int):
        q, last = lb + 1, None
        while q < rb:
            last = q
            q = self._stmt_end(q)
        return last


def lex_fragment(text: str) -> list[Tok]:
    out, i, n = [], 0, len(text)
    while i < n:
        m = _TOKEN_RE.match(text, i)
        if not m:
            out.append(Tok("punct", text[i], 0))
            i += 1
            continue
        out.append(Tok(m.lastgroup, m.group(), 0))
        i = m.end()
    return out


# ---------------------------------------------------------------- translation units

_INCLUDE_RE = re.compile(r'\s*#\s*include\s*"([^"]+)"')


def _project_headers(path: str, project: str, incdirs: list[str], seen: list[str]):
    """Quoted includes of `path` that resolve inside the project or one of the
    include directories given to the converter, depth first."""
    try:
        src = open(path).read()
    except OSError:
        return
    for line in src.splitlines():
        m = _INCLUDE_RE.match(line)
        if not m:
            continue
        name = m.group(1)
        for d in [os.path.dirname(path)] + incdirs:
            cand = os.path.realpath(os.path.join(d, name))
            if os.path.isfile(cand):
                mine = cand.startswith(project + os.sep) or any(cand.startswith(x + os.sep) for x in incdirs)
                if mine and cand not in seen:
                    _project_headers(cand, project, incdirs, seen)
                    seen.append(cand)
                break


def convert_tu(source: str, opts: Options, project: str | None = None, incdirs=(), syms: Symbols | None = None):
    """Convert one translation unit.  Returns {input path: converted text} for
    the source (key: the source path) and every project header it includes."""
    source = os.path.realpath(source)
    project = os.path.realpath(project or os.path.dirname(source))
    incdirs = [os.path.realpath(d) for d in incdirs]
    headers: list[str] = []
    _project_headers(source, project, incdirs, headers)
    syms = syms or Symbols()
    out = {}
    units = []
    for path in headers + [source]:
        u = Unit(open(path).read(), path, syms, opts, is_header=path != source)
        u.convert()
        units.append(u)
    for u in units:
        u.finish()
    for u in units:
        text = u.render()
        head = '#include "global_vars.cuh"\n'
        if opts.malloc_version > 0:
            head = "#define GPUMPI_MALLOC_V%d\n" % opts.malloc_version + head
        out[u.path] = head + text
    return out


def convert_source(text: str, opts: Options | None = None, path: str = "<input>.c") -> str:
    """Convert C source text with no project headers (tests, stdin)."""
    opts = opts or Options()
    syms = Symbols()
    u = Unit(text, path, syms, opts, is_header=False)
    u.convert()
    u.finish()
    head = '#include "global_vars.cuh"\n'
    if opts.malloc_version > 0:
        head = "#define GPUMPI_MALLOC_V%d\n" % opts.malloc_version + head
    return head + u.render()


def output_name(path: str, source: str) -> str:
    """foo.c -> foo.cu for the source; headers get `.cuh` appended."""
    if path == os.path.realpath(source):
        base, _ = os.path.splitext(path)
        return base + ".cu"
    return path + ".cuh"


def main(argv=None) -> int:
    import argparse

    ap = argparse.ArgumentParser(description="Convert C MPI programs for the device MPI runtime.")
    ap.add_argument("sources", nargs="+")
    ap.add_argument("--max-ranks", type=int,
                    default=int(os.environ.get("GPU_MPI_MAX_RANKS", DEFAULT_MAX_RANKS)))
    ap.add_argument("--malloc-version", "--malloc_version", type=int, default=0)
    ap.add_argument("--project", default=os.environ.get("GPU_MPI_PROJECT"))
    ap.add_argument("-I", dest="incdirs", action="append", default=[])
    ap.add_argument("--outdir", help="write outputs under this directory, mirroring the project tree")
    ap.add_argument("--write-to-stdout", "--write_to_stdout", action="store_true")
    a = ap.parse_args(argv)
    if a.max_ranks <= 0:
        print("ERROR: --max-ranks must be positive", file=sys.stderr)
        return 1
    opts = Options(max_ranks=a.max_ranks, malloc_version=a.malloc_version)
    for src in a.sources:
        project = os.path.realpath(a.project or os.path.dirname(os.path.abspath(src)))
        try:
            res = convert_tu(src, opts, project, a.incdirs)
        except ConvertError as e:
            print("ERROR: %s" % e, file=sys.stderr)
            return 1
        for path, text in res.items():
            if a.write_to_stdout:
                if path == os.path.realpath(src):
                    sys.stdout.write(text)
                continue
            dst = output_name(path, src)
            if a.outdir and dst.startswith(project + os.sep):
                # headers found through -I outside the project are written beside the original
                dst = os.path.join(a.outdir, os.path.relpath(dst, project))
                os.makedirs(os.path.dirname(dst), exist_ok=True)
            with open(dst, "w") as f:
                f.write(text)
    return 0


if __name__ == "__main__":
    sys.exit(main())
