"""Validated configuration models with YAML / JSON round trips.

The reference's managers and configs are pydantic models whose
``from_yaml`` / ``to_yaml`` / ``from_json`` / ``to_json`` come from one base
class (``pydantic_models/custom_types.py:18-128``).  Neither pydantic nor a
YAML library is available on every machine this package runs on, so this
module provides the same behaviour in plain Python:

* ``ConfigModel`` -- declared fields (class annotations + defaults), keyword
  construction, unknown keys rejected (the reference's ``extra="forbid"``),
  numbers coerced to the declared float/int type, nested models built from
  dicts, range / choice / length constraints from ``Field(...)``, an optional
  ``validate(self)`` hook run after construction, ``model_dump()`` without the
  excluded (tensor) fields, and the four file round trips.
* ``ValidationError`` (a ``ValueError``) with pydantic-like messages
  ("Input should be greater than or equal to 0", ...).
* ``yaml_load`` / ``yaml_dump`` -- the block-style YAML subset the reference's
  example configurations use: nested mappings and "- item" sequences,
  ``key: value`` scalars (null / true / false / numbers / quoted or plain
  strings), flow lists ``[a, b]`` and ``#`` comments.
"""

from __future__ import annotations

import json
import os
import typing
from typing import Any, Literal, Optional, Union, get_args, get_origin


class ValidationError(ValueError):
    """Invalid configuration value (a ValueError, as pydantic's is)."""


class _Unset:
    def __repr__(self):
        return "<required>"


REQUIRED = _Unset()


class FieldSpec:
    def __init__(self, default=REQUIRED, *, ge=None, gt=None, le=None, lt=None, min_length=None, max_length=None,
                 exclude=False, default_factory=None):
        self.default = default
        self.default_factory = default_factory
        self.ge, self.gt, self.le, self.lt = ge, gt, le, lt
        self.min_length, self.max_length = min_length, max_length
        self.exclude = exclude

    def make_default(self):
        if self.default_factory is not None:
            return self.default_factory()
        return self.default


def Field(default=REQUIRED, **kw) -> Any:  # noqa: N802 (mirrors pydantic.Field)
    return FieldSpec(default, **kw)


def _is_model(tp) -> bool:
    return isinstance(tp, type) and issubclass(tp, ConfigModel)


def _coerce(name: str, tp, value):
    """Check / convert ``value`` against the annotation ``tp``."""
    if tp is Any:
        return value
    origin = get_origin(tp)
    if origin is Union or (origin is not None and str(origin) == "types.UnionType"):
        args = get_args(tp)
        if value is None and type(None) in args:
            return None
        errors = []
        for a in args:
            if a is type(None):
                continue
            try:
                return _coerce(name, a, value)
            except (ValidationError, TypeError) as e:
                errors.append(str(e))
        raise ValidationError(f"{name}: value {value!r} matches none of {args} ({'; '.join(errors)})")
    if origin is Literal:
        if value not in get_args(tp):
            raise ValidationError(f"{name}: Input should be one of {get_args(tp)}, got {value!r}")
        return value
    if origin in (list, tuple):
        if not isinstance(value, (list, tuple)):
            raise ValidationError(f"{name}: Input should be a valid list, got {value!r}")
        args = get_args(tp)
        if origin is tuple and args and args[-1] is not Ellipsis:
            if len(value) != len(args):
                raise ValidationError(f"{name}: expected {len(args)} items, got {len(value)}")
            return tuple(_coerce(name, a, v) for a, v in zip(args, value))
        inner = args[0] if args else Any
        out = [_coerce(name, inner, v) for v in value]
        return tuple(out) if origin is tuple else out
    if origin is dict:
        if not isinstance(value, dict):
            raise ValidationError(f"{name}: Input should be a valid dictionary, got {value!r}")
        kt, vt = get_args(tp) or (Any, Any)
        return {_coerce(name, kt, k): _coerce(name, vt, v) for k, v in value.items()}
    if _is_model(tp):
        if isinstance(value, tp):
            return value
        if isinstance(value, dict):
            return tp(**value)
        raise ValidationError(f"{name}: expected a mapping for {tp.__name__}, got {value!r}")
    if tp is bool:
        if isinstance(value, bool):
            return value
        raise ValidationError(f"{name}: Input should be a valid boolean, got {value!r}")
    if tp is float:
        if isinstance(value, bool) or not isinstance(value, (int, float)):
            raise ValidationError(f"{name}: Input should be a valid number, got {value!r}")
        return float(value)
    if tp is int:
        if isinstance(value, bool) or not (isinstance(value, int) or (isinstance(value, float) and value.is_integer())):
            raise ValidationError(f"{name}: Input should be a valid integer, got {value!r}")
        return int(value)
    if tp is str:
        if not isinstance(value, (str, os.PathLike)):
            raise ValidationError(f"{name}: Input should be a valid string, got {value!r}")
        return os.fspath(value)
    if isinstance(tp, type):
        if isinstance(value, tp):
            return value
        raise ValidationError(f"{name}: expected {tp.__name__}, got {type(value).__name__}")
    return value


def _check_constraints(name: str, spec: FieldSpec, value):
    if value is None:
        return
    if spec.ge is not None and value < spec.ge:
        raise ValidationError(f"{name}: Input should be greater than or equal to {spec.ge}")
    if spec.gt is not None and value <= spec.gt:
        raise ValidationError(f"{name}: Input should be greater than {spec.gt}")
    if spec.le is not None and value > spec.le:
        raise ValidationError(f"{name}: Input should be less than or equal to {spec.le}")
    if spec.lt is not None and value >= spec.lt:
        raise ValidationError(f"{name}: Input should be less than {spec.lt}")
    if spec.min_length is not None and len(value) < spec.min_length:
        raise ValidationError(f"{name}: should have at least {spec.min_length} items")
    if spec.max_length is not None and len(value) > spec.max_length:
        raise ValidationError(f"{name}: should have at most {spec.max_length} items")


class ConfigModel:
    """Base class: declare fields as annotated class attributes."""

    __fields__: dict = {}

    def __init_subclass__(cls, **kw):
        super().__init_subclass__(**kw)
        hints = typing.get_type_hints(cls)
        fields = {}
        for base in reversed(cls.__bases__):  # inherited fields keep their specs
            fields.update(getattr(base, "__fields__", {}))
        for name in cls.__dict__.get("__annotations__", {}):
            if name.startswith("_") or name == "__fields__":
                continue
            tp = hints.get(name, Any)
            if get_origin(tp) is typing.ClassVar:
                continue
            raw = cls.__dict__.get(name, REQUIRED)
            if raw is REQUIRED and name in fields:  # re-annotated without a default
                raw = fields[name][1]
            spec = raw if isinstance(raw, FieldSpec) else FieldSpec(raw)
            fields[name] = (tp, spec)
        cls.__fields__ = fields
        for name, (_, spec) in fields.items():  # defaults live in __fields__, not on the class
            if name in cls.__dict__ and isinstance(cls.__dict__[name], FieldSpec):
                delattr(cls, name)

    def __init__(self, **data):
        unknown = set(data) - set(self.__fields__)
        if unknown:
            raise ValidationError(f"{type(self).__name__}: Extra inputs are not permitted: {sorted(unknown)}")
        for name, (tp, spec) in self.__fields__.items():
            if name in data:
                value = _coerce(name, tp, data[name])
                _check_constraints(name, spec, value)
            else:  # defaults are not validated (as pydantic)
                default = spec.make_default()
                if default is REQUIRED:
                    raise ValidationError(f"{type(self).__name__}: field '{name}' is required")
                value = default() if (isinstance(default, type) and _is_model(default)) else default
                if isinstance(value, ConfigModel):
                    value = type(value)(**value.model_dump())  # no shared mutable defaults
                elif isinstance(value, (list, dict)):
                    value = type(value)(value)
            object.__setattr__(self, name, value)
        self.validate()

    def validate(self) -> None:
        """Cross-field checks (override); raise ValidationError."""

    def __setattr__(self, name, value):
        if name in self.__fields__:
            tp, spec = self.__fields__[name]
            value = _coerce(name, tp, value)
            _check_constraints(name, spec, value)
        object.__setattr__(self, name, value)

    def model_dump(self) -> dict:
        out = {}
        for name, (_, spec) in self.__fields__.items():
            if spec.exclude:
                continue
            out[name] = _dump(getattr(self, name))
        return out

    def __repr__(self):
        body = ", ".join(f"{k}={getattr(self, k)!r}" for k, (_, s) in self.__fields__.items() if not s.exclude)
        return f"{type(self).__name__}({body})"

    def __eq__(self, other):
        return type(self) is type(other) and self.model_dump() == other.model_dump()

    @classmethod
    def from_yaml(cls, yaml_path, *args, **kwargs):
        with open(yaml_path, encoding="utf-8") as f:
            data = yaml_load(f.read())
        return cls(*args, **(data or {}), **kwargs)

    @classmethod
    def from_json(cls, json_path, *args, **kwargs):
        with open(json_path, encoding="utf-8") as f:
            data = json.load(f)
        return cls(*args, **data, **kwargs)

    def to_yaml(self, yaml_path) -> None:
        with open(yaml_path, "w", encoding="utf-8") as f:
            f.write(yaml_dump(self.model_dump()))

    def to_json(self, json_path) -> None:
        with open(json_path, "w", encoding="utf-8") as f:
            json.dump(self.model_dump(), f)


def _dump(v):
    if isinstance(v, ConfigModel):
        return v.model_dump()
    if isinstance(v, tuple):
        return [_dump(x) for x in v]
    if isinstance(v, list):
        return [_dump(x) for x in v]
    if isinstance(v, dict):
        return {k: _dump(x) for k, x in v.items()}
    return v


# ---------------------------------------------------------------------------
# YAML subset
# ---------------------------------------------------------------------------


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


def _scalar(text: str):
    t = text.strip()
    if t == "" or t in ("null", "Null", "NULL", "~"):
        return None
    if t in ("true", "True", "TRUE"):
        return True
    if t in ("false", "False", "FALSE"):
        return False
    if len(t) >= 2 and t[0] == t[-1] and t[0] in "'\"":
        return t[1:-1]
    if t.startswith("[") and t.endswith("]"):
        inner = t[1:-1].strip()
        return [] if not inner else [_scalar(p) for p in _split_flow(inner)]
    if t.startswith("{") and t.endswith("}"):
        inner = t[1:-1].strip()
        out = {}
        for p in _split_flow(inner) if inner else []:
            k, _, v = p.partition(":")
            out[_scalar(k)] = _scalar(v)
        return out
    try:
        return int(t)
    except ValueError:
        pass
    try:
        return float(t)
    except ValueError:
        pass
    if t in (".inf", ".Inf"):
        return float("inf")
    if t in ("-.inf", "-.Inf"):
        return float("-inf")
    return t


def _split_flow(s: str) -> list[str]:
    parts, depth, cur, quote = [], 0, [], None
    for ch in s:
        if quote:
            cur.append(ch)
            if ch == quote:
                quote = None
            continue
        if ch in "'\"":
            quote = ch
        elif ch in "[{":
            depth += 1
        elif ch in "]}":
            depth -= 1
        elif ch == "," and depth == 0:
            parts.append("".join(cur).strip())
            cur = []
            continue
        cur.append(ch)
    if "".join(cur).strip():
        parts.append("".join(cur).strip())
    return parts


def yaml_load(text: str):
    """Parse the block-style YAML subset described in the module docstring."""
    lines = []
    for raw in text.splitlines():
        if raw.strip() in ("---", "..."):
            continue
        s = _strip_comment(raw)
        if s.strip():
            lines.append((len(s) - len(s.lstrip(" ")), s.strip()))
    pos = 0

    def parse_block(indent):
        nonlocal pos
        if pos >= len(lines):
            return None
        if lines[pos][1].startswith("- ") or lines[pos][1] == "-":
            seq = []
            while pos < len(lines) and lines[pos][0] == indent and (lines[pos][1].startswith("- ")
                                                                    or lines[pos][1] == "-"):
                body = lines[pos][1][1:].strip()
                pos += 1
                if not body:
                    seq.append(parse_block(lines[pos][0]) if pos < len(lines) and lines[pos][0] > indent else None)
                elif ":" in body and not body.startswith(("'", '"', "[", "{")) and _is_key(body):
                    # "- key: value" starts a mapping inside the sequence item
                    lines.insert(pos, (indent + 2, body))
                    seq.append(parse_block(indent + 2))
                else:
                    seq.append(_scalar(body))
            return seq
        mapping = {}
        while pos < len(lines) and lines[pos][0] == indent:
            body = lines[pos][1]
            if not _is_key(body):
                raise ValueError(f"YAML: cannot parse line {body!r}")
            key, _, rest = body.partition(":")
            key = _scalar(key)
            pos += 1
            if rest.strip():
                mapping[key] = _scalar(rest)
            elif pos < len(lines) and (lines[pos][0] > indent or (lines[pos][0] == indent
                                                                   and lines[pos][1].startswith("-"))):
                mapping[key] = parse_block(lines[pos][0])
            else:
                mapping[key] = None
        return mapping

    if not lines:
        return None
    out = parse_block(lines[0][0])
    if pos != len(lines):
        raise ValueError(f"YAML: unexpected indentation at {lines[pos][1]!r}")
    return out


def _is_key(body: str) -> bool:
    key, sep, rest = body.partition(":")
    return bool(sep) and (rest == "" or rest.startswith(" ")) and bool(key.strip())


def _fmt_scalar(v) -> str:
    if v is None:
        return "null"
    if v is True:
        return "true"
    if v is False:
        return "false"
    if isinstance(v, (int, float)):
        return repr(v)
    s = str(v)
    if s == "" or s.strip() != s or any(c in s for c in ":#[]{},'\"") or _scalar(s) != s:
        return json.dumps(s)
    return s


def yaml_dump(data, indent: int = 0) -> str:
    pad = " " * indent
    out = []
    if isinstance(data, dict):
        for k, v in data.items():
            if isinstance(v, dict) and v:
                out.append(f"{pad}{k}:")
                out.append(yaml_dump(v, indent + 2))
            elif isinstance(v, list) and v and any(isinstance(x, (dict, list)) for x in v):
                out.append(f"{pad}{k}:")
                out.append(yaml_dump(v, indent + 2))
            elif isinstance(v, list):
                out.append(f"{pad}{k}: [{', '.join(_fmt_scalar(x) for x in v)}]")
            elif isinstance(v, dict):
                out.append(f"{pad}{k}: {{}}")
            else:
                out.append(f"{pad}{k}: {_fmt_scalar(v)}")
    elif isinstance(data, list):
        for v in data:
            if isinstance(v, (dict, list)):
                sub = yaml_dump(v, indent + 2).splitlines()
                out.append(f"{pad}- {sub[0].strip()}")
                out.extend(sub[1:])
            else:
                out.append(f"{pad}- {_fmt_scalar(v)}")
    else:
        out.append(pad + _fmt_scalar(data))
    return "\n".join(x for x in out if x != "") + ("\n" if indent == 0 else "")


__all__ = ["ConfigModel", "Field", "ValidationError", "Optional", "yaml_load", "yaml_dump"]
