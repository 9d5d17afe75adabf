"""A YAML subset for run configurations (no YAML library is available).

Covers what the reference's setup files use (setups/*.yaml, read by
serde_yaml at src/app.rs:308): nested block mappings by indentation,
`key: value` scalars, `~` / `null` for None, booleans, integers, floats
(including `1e3` and `.inf`), and plain or quoted strings; `#` comments.
Flow collections, sequences, anchors and multi-line scalars are rejected.
"""
import math
import re

_INT = re.compile(r"^[-+]?[0-9]+$")
_FLOAT = re.compile(r"^[-+]?(\.[0-9]+|[0-9]+(\.[0-9]*)?)([eE][-+]?[0-9]+)?$")


class YamlError(ValueError):
    pass


def parse_scalar(text: str):
    s = text.strip()
    if s in ("~", "null", "Null", "NULL", ""):
        return None
    if s in ("true", "True", "TRUE"):
        return True
    if s in ("false", "False", "FALSE"):
        return False
    if len(s) >= 2 and s[0] == s[-1] and s[0] in "'\"":
        return s[1:-1]
    if _INT.match(s):
        return int(s)
    if _FLOAT.match(s):
        return float(s)
    if s in (".inf", "+.inf"):
        return math.inf
    if s == "-.inf":
        return -math.inf
    if s in (".nan", ".NaN"):
        return math.nan
    if s[0] in "[{&*!|>":
        raise YamlError("unsupported YAML construct: %r" % s)
    return s


def _strip_comment(line: str) -> str:
    out, quote = [], None
    for i, ch in enumerate(line):
        if quote:
            if ch == quote:
                quote = None
        elif ch in "'\"":
            quote = ch
        elif ch == "#" and (i == 0 or line[i - 1] in " \t"):
            break
        out.append(ch)
    return "".join(out).rstrip()


def loads(text: str) -> dict:
    """Parse a block-mapping YAML document into nested dicts."""
    root: dict = {}
    stack = [(-1, root)]          # (indent, mapping)
    pending = None                # (indent, parent, key) awaiting a nested mapping
    for lineno, raw in enumerate(text.splitlines(), 1):
        line = _strip_comment(raw)
        if not line.strip() or line.strip() == "---":
            continue
        if "\t" in line[: len(line) - len(line.lstrip())]:
            raise YamlError("line %d: tabs in indentation" % lineno)
        indent = len(line) - len(line.lstrip(" "))
        body = line.strip()
        if body.startswith("- "):
            raise YamlError("line %d: sequences are not supported" % lineno)
        m = re.match(r"^([^:]+?)\s*:(\s+(.*))?$", body)
        if not m:
            raise YamlError("line %d: expected `key: value`" % lineno)
        key, value = m.group(1).strip(), m.group(3)
        if pending is not None:
            p_indent, p_parent, p_key = pending
            if indent > p_indent:
                child: dict = {}
                p_parent[p_key] = child
                stack.append((p_indent, child))
            else:
                p_parent[p_key] = None
            pending = None
        while len(stack) > 1 and indent <= stack[-1][0]:
            stack.pop()
        parent = stack[-1][1]
        if key in parent:
            raise YamlError("line %d: duplicate key %r" % (lineno, key))
        if value is None or value == "":
            pending = (indent, parent, key)
            parent[key] = None
        else:
            parent[key] = parse_scalar(value)
    return root


def _fmt(v) -> str:
    if v is None:
        return "~"
    if isinstance(v, bool):
        return "true" if v else "false"
    if isinstance(v, float):
        if math.isinf(v):
            return ".inf" if v > 0 else "-.inf"
        return repr(v)
    return str(v)


def dumps(d: dict, indent: int = 0) -> str:
    out = []
    for k, v in d.items():
        if isinstance(v, dict):
            out.append(" " * indent + "%s:" % k)
            out.append(dumps(v, indent + 2))
        else:
            out.append(" " * indent + "%s: %s" % (k, _fmt(v)))
    return "\n".join(x for x in out if x)
