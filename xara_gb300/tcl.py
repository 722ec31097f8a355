"""A Tcl subset for the reference's model scripts, run on the device path.

The reference reads Tcl scripts (its interpreter registers ``model``,
``node``, ``element``, ``analyze`` ... as Tcl commands).  This image has no
Tcl, so this module evaluates the part of Tcl such scripts use and hands
every other command to :mod:`xara_gb300.openseespy`::

    from xara_gb300 import tcl
    tcl.eval_script(open("frame.tcl").read())
    tcl.eval_script("puts [nodeDisp 7 1]")

Supported: words separated by blanks, ``{}`` grouping (no substitution),
``""`` grouping, ``$name`` / ``${name}`` and ``[command]`` substitution,
backslash-newline, ``#`` comments, ``;``; the commands ``set``, ``unset``,
``incr``, ``expr`` (arithmetic, comparisons, ``&& || !``, ``? :`` and the
math functions), ``if/elseif/else``, ``for``, ``foreach``, ``while``,
``break``, ``continue``, ``proc``/``return``, ``puts``, ``list``,
``llength``, ``lindex``, ``lappend``, ``source``.  Numbers reach the model
commands as numbers, flags (``-ndm``, ``-time`` ...) as strings.
"""
import math
import re

from . import openseespy as ops


class TclError(Exception):
    pass


class _Break(Exception):
    pass


class _Continue(Exception):
    pass


class _Return(Exception):
    def __init__(self, value):
        super().__init__()
        self.value = value


def _number(tok):
    """A token as the model commands want it: int, float or the string."""
    if not isinstance(tok, str):
        return tok
    try:
        return int(tok)
    except ValueError:
        pass
    try:
        return float(tok)
    except ValueError:
        return tok


def _fmt(v):
    """Tcl's string form of a value."""
    if isinstance(v, bool):
        return "1" if v else "0"
    if isinstance(v, float):
        r = repr(v)
        return r[:-2] if r.endswith(".0") and abs(v) < 1e16 else r
    if isinstance(v, (list, tuple)):
        return " ".join(_quote(_fmt(x)) for x in v)
    return str(v)


def _quote(s):
    return "{" + s + "}" if (not s or any(c.isspace() for c in s)) else s


class _I(int):
    """An integer of an expression: division of two integers floors, as in Tcl."""

    def _wrap(self, v):
        return _I(v) if isinstance(v, int) and not isinstance(v, bool) else v

    def __truediv__(self, o):
        if isinstance(o, int):
            return _I(int(self) // int(o))
        return int(self) / o

    def __rtruediv__(self, o):
        if isinstance(o, int):
            return _I(int(o) // int(self))
        return o / int(self)

    def __add__(self, o):
        return self._wrap(int(self) + o)

    __radd__ = __add__

    def __sub__(self, o):
        return self._wrap(int(self) - o)

    def __rsub__(self, o):
        return self._wrap(o - int(self))

    def __mul__(self, o):
        return self._wrap(int(self) * o)

    __rmul__ = __mul__

    def __mod__(self, o):
        return self._wrap(int(self) % o)

    def __neg__(self):
        return _I(-int(self))


def _ternary(e):
    """cond ? a : b (right-associative, outside parentheses) as Python."""
    depth, q = 0, -1
    for k, c in enumerate(e):
        depth += {"(": 1, ")": -1}.get(c, 0)
        if c == "?" and depth == 0:
            q = k
            break
    if q < 0:
        return e
    depth, nest = 0, 0
    for k in range(q + 1, len(e)):
        c = e[k]
        depth += {"(": 1, ")": -1}.get(c, 0)
        if depth == 0 and c == "?":
            nest += 1
        elif depth == 0 and c == ":":
            if nest == 0:
                return (f"(({_ternary(e[q + 1:k])}) if ({e[:q]}) "
                        f"else ({_ternary(e[k + 1:])}))")
            nest -= 1
    raise TclError(f"expr {e!r}: '?' without ':'")


def _is_body(word):
    """A script argument (several words, a newline, or empty), not a number
    or a flag."""
    return isinstance(word, str) and (not word.strip() or any(c.isspace() for c in word.strip()))


_INT_LITERAL = re.compile(r"(?<![\w.])(\d+)(?![\w.])")

_MATH = {n: getattr(math, n) for n in ("sqrt", "sin", "cos", "tan", "asin", "acos", "atan",
                                        "atan2", "exp", "log", "log10", "pow", "sinh", "cosh",
                                        "tanh", "floor", "ceil", "hypot", "fmod")}
_MATH.update(abs=abs, int=lambda x: int(x), double=float, round=lambda x: int(round(x)),
             min=min, max=max, pi=math.pi)


class Interp:
    def __init__(self):
        self.frames = [{}]
        self.procs = {}
        self.out = []                      # what puts printed (also printed)

    # -- variables -----------------------------------------------------------
    @property
    def vars(self):
        return self.frames[-1]

    def getvar(self, name):
        m = re.fullmatch(r"(\w+)\((.*)\)", name)
        if m:
            name = f"{m.group(1)}({m.group(2)})"
        if name not in self.vars:
            raise TclError(f"can't read \"{name}\": no such variable")
        return self.vars[name]

    # -- parsing -------------------------------------------------------------
    def eval(self, script):
        result = ""
        for words in self._commands(script):
            if words:
                result = self.call(words)
        return result

    def _commands(self, script):
        """Commands of a script, each a list of substituted words."""
        i, n = 0, len(script)
        while i < n:
            # skip blanks, newlines and semicolons between commands
            while i < n and (script[i] in " \t\r\n;"):
                i += 1
            if i >= n:
                break
            if script[i] == "#":
                while i < n and script[i] != "\n":
                    if script[i] == "\\" and i + 1 < n:
                        i += 1
                    i += 1
                continue
            words = []
            while i < n and script[i] not in "\n;":
                if script[i] in " \t\r":
                    i += 1
                    continue
                if script[i] == "\\" and i + 1 < n and script[i + 1] == "\n":
                    i += 2
                    continue
                word, i = self._word(script, i)
                words.append(word)
            yield words

    def _word(self, s, i):
        if s[i] == "{":
            depth, j = 1, i + 1
            while j < len(s) and depth:
                if s[j] == "\\":
                    j += 2
                    continue
                depth += {"{": 1, "}": -1}.get(s[j], 0)
                j += 1
            if depth:
                raise TclError("missing close-brace")
            return s[i + 1:j - 1], j
        if s[i] == '"':
            j = i + 1
            parts = []
            while j < len(s) and s[j] != '"':
                j = self._subst_one(s, j, parts)
            if j >= len(s):
                raise TclError("missing \"")
            return "".join(_fmt(p) for p in parts), j + 1
        parts = []
        j = i
        while j < len(s) and s[j] not in " \t\r\n;":
            j = self._subst_one(s, j, parts)
        if len(parts) == 1 and not isinstance(parts[0], str):
            return parts[0], j
        return "".join(_fmt(p) for p in parts), j

    def _subst_one(self, s, j, parts):
        c = s[j]
        if c == "$":
            m = re.match(r"\$(\{([^}]*)\}|(\w+)(\([^)]*\))?)", s[j:])
            if not m:
                parts.append("$")
                return j + 1
            name = m.group(2) if m.group(2) is not None else m.group(3)
            if m.group(4):
                idx = self.subst(m.group(4)[1:-1])
                name = f"{name}({idx})"
            parts.append(self.getvar(name))
            return j + len(m.group(0))
        if c == "[":
            depth, k = 1, j + 1
            while k < len(s) and depth:
                if s[k] == "\\":
                    k += 2
                    continue
                depth += {"[": 1, "]": -1}.get(s[k], 0)
                k += 1
            parts.append(self.eval(s[j + 1:k - 1]))
            return k
        if c == "\\" and j + 1 < len(s):
            parts.append({"n": "\n", "t": "\t"}.get(s[j + 1], s[j + 1]))
            return j + 2
        parts.append(c)
        return j + 1

    def subst(self, s):
        parts, j = [], 0
        while j < len(s):
            j = self._subst_one(s, j, parts)
        return "".join(_fmt(p) for p in parts)

    # -- expressions ---------------------------------------------------------
    def expr(self, text):
        s = self.subst(text) if ("$" in text or "[" in text) else text
        py = s.replace("&&", " and ").replace("||", " or ")
        py = re.sub(r"!(?!=)", " not ", py)
        py = _ternary(py)
        py = _INT_LITERAL.sub(r"_I(\1)", py)
        try:
            v = eval(py, {"__builtins__": {}}, dict(_MATH, _I=_I))  # noqa: S307 - the user's script
        except Exception as e:
            raise TclError(f"expr {text!r}: {e}") from None
        if isinstance(v, bool):
            return int(v)
        return int(v) if isinstance(v, int) else v

    def truth(self, text):
        return bool(self.expr(text))

    # -- commands ------------------------------------------------------------
    def call(self, words):
        name, args = _fmt(words[0]), words[1:]
        fn = getattr(self, "_cmd_" + name, None)
        if fn is not None:
            return fn(*args)
        if name in self.procs:
            return self._call_proc(name, args)
        target = getattr(ops, name, None)
        if target is None or name.startswith("_") or not callable(target):
            raise TclError(f"invalid command name \"{name}\"")
        r = target(*[_number(a) for a in args])
        return "" if r is None else r

    # model commands whose last word is a script (section Fiber tag {...},
    # pattern Plain tag series {...}) or a list (timeSeries Path -values {...})
    def _cmd_section(self, kind, tag, *rest):
        rest = list(rest)
        body = rest.pop() if rest and _is_body(rest[-1]) else None
        ops.section(_fmt(kind), _number(tag), *[_number(a) for a in rest])
        if body is not None:
            self.eval(body)
        return ""

    def _cmd_pattern(self, kind, tag, *rest):
        rest = list(rest)
        body = rest.pop() if rest and _is_body(rest[-1]) else None
        if _fmt(kind) == "Plain" and rest and isinstance(_number(rest[0]), str):
            # an inline series: pattern Plain tag Linear {...}
            ts = -int(_number(tag))
            ops.timeSeries(_fmt(rest[0]), ts, *[_number(a) for a in rest[1:]])
            rest = [ts]
        ops.pattern(_fmt(kind), _number(tag), *[_number(a) for a in rest])
        if body is not None:
            self.eval(body)
        return ""

    def _cmd_timeSeries(self, kind, tag, *rest):
        args = []
        for a in rest:
            if isinstance(a, str) and " " in a.strip():
                args.extend(_number(x) for x in self._split(a))
            else:
                args.append(_number(a))
        ops.timeSeries(_fmt(kind), _number(tag), *args)
        return ""

    def _cmd_set(self, name, *value):
        if value:
            self.vars[_fmt(name)] = value[0]
        return self.getvar(_fmt(name))

    def _cmd_unset(self, *names):
        for n in names:
            self.vars.pop(_fmt(n), None)
        return ""

    def _cmd_incr(self, name, by=1):
        v = int(_number(self.vars.get(name, 0))) + int(_number(by))
        self.vars[name] = v
        return v

    def _cmd_expr(self, *parts):
        return self.expr(" ".join(_fmt(p) for p in parts))

    def _cmd_puts(self, *args):
        text = _fmt(args[-1]) if args else ""
        print(text)
        self.out.append(text)
        return ""

    def _cmd_if(self, cond, *rest):
        rest = list(rest)
        if rest and rest[0] == "then":
            rest.pop(0)
        if self.truth(cond):
            return self.eval(rest[0])
        rest = rest[1:]
        while rest:
            kw = rest.pop(0)
            if kw == "elseif":
                c, body = rest.pop(0), rest.pop(0)
                if rest and rest[0] == "then":
                    rest.pop(0)
                if self.truth(c):
                    return self.eval(body)
            elif kw == "else":
                return self.eval(rest.pop(0))
            else:
                return self.eval(kw)
        return ""

    def _loop_body(self, body):
        try:
            self.eval(body)
        except _Continue:
            pass

    def _cmd_for(self, init, cond, step, body):
        self.eval(init)
        try:
            while self.truth(cond):
                self._loop_body(body)
                self.eval(step)
        except _Break:
            pass
        return ""

    def _cmd_while(self, cond, body):
        try:
            while self.truth(cond):
                self._loop_body(body)
        except _Break:
            pass
        return ""

    def _cmd_foreach(self, var, items, body):
        names = self._split(_fmt(var))
        vals = self._split(_fmt(items))
        try:
            for k in range(0, len(vals), len(names)):
                for n, v in zip(names, vals[k:k + len(names)]):
                    self.vars[n] = v
                self._loop_body(body)
        except _Break:
            pass
        return ""

    def _cmd_break(self):
        raise _Break()

    def _cmd_continue(self):
        raise _Continue()

    def _cmd_proc(self, name, params, body):
        self.procs[_fmt(name)] = (self._split(_fmt(params)), body)
        return ""

    def _call_proc(self, name, args):
        params, body = self.procs[name]
        frame = {}
        for k, p in enumerate(params):
            pp = self._split(p)
            if pp[0] == "args":
                frame["args"] = list(args[k:])
                break
            frame[pp[0]] = args[k] if k < len(args) else (pp[1] if len(pp) > 1 else "")
        self.frames.append(frame)
        try:
            return self.eval(body)
        except _Return as r:
            return r.value
        finally:
            self.frames.pop()

    def _cmd_return(self, value=""):
        raise _Return(value)

    def _cmd_list(self, *items):
        return _fmt([_fmt(i) for i in items])

    def _cmd_llength(self, lst):
        return len(self._split(_fmt(lst)))

    def _cmd_lindex(self, lst, idx):
        items = self._split(_fmt(lst))
        k = len(items) - 1 if _fmt(idx) == "end" else int(_number(idx))
        return items[k] if 0 <= k < len(items) else ""

    def _cmd_lappend(self, name, *items):
        cur = self._split(_fmt(self.vars.get(name, "")))
        self.vars[name] = _fmt(cur + [_fmt(i) for i in items])
        return self.vars[name]

    def _cmd_source(self, path):
        with open(_fmt(path)) as f:
            return self.eval(f.read())

    def _split(self, s):
        """A Tcl list's elements."""
        out, i = [], 0
        while i < len(s):
            while i < len(s) and s[i].isspace():
                i += 1
            if i >= len(s):
                break
            if s[i] == "{":
                w, i = self._word(s, i)
                out.append(w)
            else:
                j = i
                while j < len(s) and not s[j].isspace():
                    j += 1
                out.append(s[i:j])
                i = j
        return out


_INTERP = Interp()


def eval_script(script, fresh=False):
    """Evaluate a script; model and analysis commands go to the device path."""
    global _INTERP
    if fresh:
        _INTERP = Interp()
    return _INTERP.eval(script)
