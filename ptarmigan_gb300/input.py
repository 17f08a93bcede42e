"""The reference's YAML input (beam, laser, control, stats, output and
constants sections; src/input/mod.rs, main.rs:339-1000): a reader for the
YAML subset those files use, and an evaluator for the arithmetic
expressions their values may hold, with the reference's built-in
constants and functions (input/mod.rs:56-140).

No third-party YAML package is needed: mappings by indentation, block
sequences ("- item"), flow sequences ("[a, b]"), scalars, quotes, comments
and a leading "---" are read; anchors, tags and multi-line scalars are not.
"""

import math

# constants.rs
ELECTRON_MASS = 9.109383e-31
PROTON_MASS = 1.672622e-27
SPEED_OF_LIGHT = 2.997925e8
ELECTRON_CHARGE = -1.602177e-19
ELEMENTARY_CHARGE = 1.602177e-19
VACUUM_PERMITTIVITY = 8.854188e-12
COMPTON_TIME = 1.28808867e-21


class InputError(ValueError):
    pass


# ------------------------------------------------------------------ YAML ---
def _strip_comment(line):
    out, q = [], None
    for ch in line:
        if q:
            if ch == q:
                q = None
        elif ch in "'\"":
            q = ch
        elif ch == "#":
            break
        out.append(ch)
    return "".join(out).rstrip()


def _scalar(s):
    s = s.strip()
    if len(s) >= 2 and s[0] == s[-1] and s[0] in "'\"":
        return s[1:-1]
    if s.startswith("[") and s.endswith("]"):
        inner = s[1:-1].strip()
        return [_scalar(x) for x in _split_flow(inner)] if inner else []
    return s


def _split_flow(s):
    parts, depth, cur, q = [], 0, [], None
    for ch in s:
        if q:
            cur.append(ch)
            if ch == q:
                q = None
            continue
        if ch in "'\"":
            q = ch
        elif ch in "([":
            depth += 1
        elif ch in ")]":
            depth -= 1
        elif ch == "," and depth == 0:
            parts.append("".join(cur))
            cur = []
            continue
        cur.append(ch)
    parts.append("".join(cur))
    return [p.strip() for p in parts]


def parse_yaml(text):
    """Nested dicts and lists of strings from the YAML subset above."""
    lines = []
    for raw in text.splitlines():
        line = _strip_comment(raw)
        if not line.strip() or line.strip() in ("---", "..."):
            continue
        if "\t" in line[:len(line) - len(line.lstrip())]:
            raise InputError("tabs are not allowed in indentation")
        lines.append((len(line) - len(line.lstrip()), line.strip()))
    pos = [0]

    def block(indent):
        if pos[0] >= len(lines):
            return None
        ind, text = lines[pos[0]]
        if text.startswith("- ") or text == "-":
            out = []
            while pos[0] < len(lines) and lines[pos[0]][0] == ind and (lines[pos[0]][1].startswith("- ") or
                                                                        lines[pos[0]][1] == "-"):
                item = lines[pos[0]][1][1:].strip()
                pos[0] += 1
                if item:
                    out.append(_scalar(item))
                else:
                    out.append(block(lines[pos[0]][0]) if pos[0] < len(lines) and lines[pos[0]][0] > ind else None)
            return out
        out = {}
        while pos[0] < len(lines) and lines[pos[0]][0] == ind:
            text = lines[pos[0]][1]
            if ":" not in text:
                raise InputError("expected 'key: value' in %r" % text)
            key, rest = text.split(":", 1)
            key, rest = key.strip(), rest.strip()
            pos[0] += 1
            if rest:
                out[key] = _scalar(rest)
            elif pos[0] < len(lines) and lines[pos[0]][0] > ind:
                out[key] = block(lines[pos[0]][0])
            elif pos[0] < len(lines) and lines[pos[0]][0] == ind and lines[pos[0]][1].startswith("- "):
                out[key] = block(ind)  # a sequence at the key's own indentation
            else:
                out[key] = None
        return out
    doc = block(lines[0][0]) if lines else {}
    if pos[0] != len(lines):
        raise InputError("could not read the input past line %r" % (lines[pos[0]][1],))
    return doc


# ------------------------------------------------------------ expressions ---
def _erf(x):
    return math.tanh(167.0 * x / 148.0 + 11.0 * x ** 3 / 109.0)


FUNCTIONS = {
    "sqrt": math.sqrt, "cbrt": lambda x: math.copysign(abs(x) ** (1.0 / 3.0), x), "abs": abs, "exp": math.exp,
    "ln": math.log, "sin": math.sin, "cos": math.cos, "tan": math.tan, "asin": math.asin, "acos": math.acos,
    "atan": math.atan, "atan2": math.atan2, "sinh": math.sinh, "cosh": math.cosh, "tanh": math.tanh,
    "asinh": math.asinh, "acosh": math.acosh, "atanh": math.atanh, "floor": math.floor, "ceil": math.ceil,
    "round": lambda x: math.floor(abs(x) + 0.5) * (1.0 if x >= 0 else -1.0),
    "signum": lambda x: math.copysign(1.0, x), "erf": _erf,
    "step": lambda x, lo, hi: 1.0 if lo <= x < hi else 0.0,
    "gauss": lambda x, mu, sigma: math.exp(-(x - mu) ** 2 / (2.0 * sigma ** 2)),
    "critical": lambda omega: VACUUM_PERMITTIVITY * ELECTRON_MASS * omega ** 2 / ELEMENTARY_CHARGE ** 2,
}


def default_context():
    """The reference's built-in constants (input/mod.rs:61-79)."""
    return {"m": ELECTRON_MASS, "me": ELECTRON_MASS, "mp": PROTON_MASS, "c": SPEED_OF_LIGHT, "e": ELECTRON_CHARGE,
            "qe": ELECTRON_CHARGE, "eV": ELEMENTARY_CHARGE, "keV": 1.0e3 * ELEMENTARY_CHARGE,
            "MeV": 1.0e6 * ELEMENTARY_CHARGE, "GeV": 1.0e9 * ELEMENTARY_CHARGE, "femto": 1.0e-15, "pico": 1.0e-12,
            "nano": 1.0e-9, "micro": 1.0e-6, "milli": 1.0e-3, "pi": math.pi, "degree": math.pi / 180.0}


class _Parser:
    """Recursive descent over + - * / % ^ (right-associative power), unary
    signs, parentheses and function calls."""

    def __init__(self, text, ctx):
        self.toks, self.i, self.ctx = self._lex(text), 0, ctx

    @staticmethod
    def _lex(s):
        toks, i = [], 0
        while i < len(s):
            ch = s[i]
            if ch.isspace():
                i += 1
            elif ch.isdigit() or (ch == "." and i + 1 < len(s) and s[i + 1].isdigit()):
                j = i
                while j < len(s) and (s[j].isdigit() or s[j] == "."):
                    j += 1
                if j < len(s) and s[j] in "eE" and (j + 1 < len(s) and (s[j + 1].isdigit() or
                                                                        (s[j + 1] in "+-" and j + 2 < len(s) and
                                                                         s[j + 2].isdigit()))):
                    j += 2
                    while j < len(s) and s[j].isdigit():
                        j += 1
                toks.append(("num", float(s[i:j])))
                i = j
            elif ch.isalpha() or ch == "_":
                j = i
                while j < len(s) and (s[j].isalnum() or s[j] == "_"):
                    j += 1
                toks.append(("id", s[i:j]))
                i = j
            elif ch in "+-*/%^(),":
                toks.append(("op", ch))
                i += 1
            else:
                raise InputError("unexpected %r in expression %r" % (ch, s))
        return toks

    def peek(self):
        return self.toks[self.i] if self.i < len(self.toks) else (None, None)

    def take(self, op=None):
        t = self.peek()
        if op is not None and t != ("op", op):
            raise InputError("expected %r" % op)
        self.i += 1
        return t

    def expr(self):
        v = self.term()
        while self.peek() in (("op", "+"), ("op", "-")):
            v = v + self.term() if self.take()[1] == "+" else v - self.term()
        return v

    def term(self):
        v = self.unary()
        while self.peek() in (("op", "*"), ("op", "/"), ("op", "%")):
            op = self.take()[1]
            r = self.unary()
            v = v * r if op == "*" else (v / r if op == "/" else math.fmod(v, r))
        return v

    def unary(self):
        if self.peek() == ("op", "-"):
            self.take()
            return -self.unary()
        if self.peek() == ("op", "+"):
            self.take()
            return self.unary()
        return self.power()

    def power(self):
        base = self.atom()
        if self.peek() == ("op", "^"):
            self.take()
            return base ** self.unary()
        return base

    def atom(self):
        kind, val = self.take()
        if kind == "num":
            return val
        if kind == "op" and val == "(":
            v = self.expr()
            self.take(")")
            return v
        if kind == "id":
            if self.peek() == ("op", "("):
                self.take()
                args = []
                if self.peek() != ("op", ")"):
                    args.append(self.expr())
                    while self.peek() == ("op", ","):
                        self.take()
                        args.append(self.expr())
                self.take(")")
                if val not in FUNCTIONS:
                    raise InputError("unknown function %r" % val)
                return float(FUNCTIONS[val](*args))
            if val in ("true", "false"):
                raise InputError("a boolean is not a number")
            if val not in self.ctx:
                raise InputError("unknown name %r" % val)
            return self.ctx[val]
        raise InputError("unexpected token %r" % (val,))

    def parse(self):
        v = self.expr()
        if self.i != len(self.toks):
            raise InputError("trailing tokens in expression")
        return float(v)


def evaluate(text, ctx):
    return _Parser(str(text), ctx).parse()


# ---------------------------------------------------------------- input ---
class Input:
    """An input file: read("laser:a0") and friends with the reference's
    conversions, expressions evaluated in the constants context."""

    def __init__(self, text):
        self.doc = parse_yaml(text) or {}
        self.ctx = default_context()
        consts = self.doc.get("constants") or {}
        for k, v in consts.items():  # in file order, each available to the next
            if isinstance(v, list) or v is None:
                raise InputError("constants:%s is not a number" % k)
            self.ctx[k] = evaluate(v, self.ctx)

    @staticmethod
    def from_file(path):
        with open(path) as f:
            return Input(f.read())

    def _get(self, path):
        node = self.doc
        for part in path.split(":"):
            if not isinstance(node, dict) or part not in node:
                return None
            node = node[part]
        return node

    def contains(self, path):
        return self._get(path) is not None

    def evaluate(self, s):
        return evaluate(s, self.ctx)

    def func(self, path, arg):
        """Input::func (input/mod.rs:180-204): the expression at `path` as a
        function of the variable `arg`, evaluated in the constants context."""
        text = self._get(path)
        if text is None or isinstance(text, (list, dict)):
            raise InputError("%s is missing" % path)

        def f(x):
            ctx = dict(self.ctx)
            ctx[arg] = float(x)
            return evaluate(text, ctx)
        return f

    def float(self, path, default=None):
        v = self._get(path)
        if v is None:
            if default is None:
                raise InputError("%s is missing" % path)
            return default
        if isinstance(v, list):
            raise InputError("%s must be a number" % path)
        return self.evaluate(v)

    def int(self, path, default=None):
        return int(round(self.float(path, None if default is None else float(default))))

    def bool(self, path, default=None):
        v = self._get(path)
        if v is None:
            if default is None:
                raise InputError("%s is missing" % path)
            return default
        if str(v).lower() in ("true", "yes", "on"):
            return True
        if str(v).lower() in ("false", "no", "off"):
            return False
        raise InputError("%s must be true or false" % path)

    def str(self, path, default=None):
        v = self._get(path)
        if v is None:
            if default is None:
                raise InputError("%s is missing" % path)
            return default
        return str(v)

    def list(self, path, default=None):
        v = self._get(path)
        if v is None:
            return [] if default is None else default
        return v if isinstance(v, list) else [v]

    def floats(self, path, default=None):
        v = self._get(path)
        if v is None:
            return default
        return [self.evaluate(x) for x in (v if isinstance(v, list) else [v])]

    def loop(self, path):
        """Input::read_loop (input/mod.rs:239-263): a value, or start, stop,
        step."""
        v = self._get(path)
        if isinstance(v, dict) and "start" in v:
            start, stop, step = (self.float(path + ":" + k) for k in ("start", "stop", "step"))
            out, x = [], start
            while x <= stop:
                out.append(x)
                x = x + step
            return out
        return [self.float(path)]
