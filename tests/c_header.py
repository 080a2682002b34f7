"""A small parser of include/bioshell_crmsd.h for the binding checks: the
exported functions (name, parameter types, return type), the structs (field
names and types, in order) and the integer constants of its enums and
#defines.  Types come back normalised ("const double *", "int32_t[6]")."""
from __future__ import annotations

import os
import re

HEADER = os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))), "include", "bioshell_crmsd.h")


def _strip_comments(text: str) -> str:
    text = re.sub(r"/\*.*?\*/", " ", text, flags=re.S)
    return re.sub(r"//[^\n]*", " ", text)


def _norm(t: str) -> str:
    t = re.sub(r"\s+", " ", t.strip())
    t = re.sub(r"\s*\*\s*", " *", t)  # "double*" / "double *" -> "double *"
    t = t.replace(" * *", " **").replace("* const", "*const")
    return t.strip()


def _split_decl(d: str):
    """'const double *xyz' -> ('const double *', 'xyz'); arrays kept on the type."""
    d = d.strip()
    m = re.match(r"^(.*?)([A-Za-z_]\w*)\s*(\[\s*\d+\s*\])?$", d)
    typ, name, arr = m.group(1), m.group(2), m.group(3)
    typ = _norm(typ)
    if arr:
        typ += "[" + re.sub(r"\D", "", arr) + "]"
    return typ, name


def functions(path: str = HEADER):
    text = _strip_comments(open(path).read())
    out = {}
    for m in re.finditer(r"BS_API\s+([^;{]*?)\b(bs_\w+)\s*\(([^)]*)\)\s*;", text, flags=re.S):
        ret = _norm(m.group(1))
        params = m.group(3).strip()
        plist = [] if params in ("", "void") else [_split_decl(p)[0] for p in params.split(",")]
        out[m.group(2)] = (ret, plist)
    return out


def structs(path: str = HEADER):
    text = _strip_comments(open(path).read())
    out = {}
    for m in re.finditer(r"typedef struct\s*\{(.*?)\}\s*(\w+)\s*;", text, flags=re.S):
        fields = [_split_decl(f) for f in m.group(1).split(";") if f.strip()]
        out[m.group(2)] = [(name, typ) for typ, name in fields]
    return out


def opaque_types(path: str = HEADER):
    text = _strip_comments(open(path).read())
    return re.findall(r"typedef struct (\w+) \1\s*;", text)


def constants(path: str = HEADER):
    text = _strip_comments(open(path).read())
    out = {}
    for body in re.findall(r"enum\s*\{(.*?)\}", text, flags=re.S):
        for name, val in re.findall(r"(BS_\w+)\s*=\s*(-?\d+)", body):
            out[name] = int(val)
    for name, val in re.findall(r"#define\s+(BS_\w+)\s+(-?\d+)\s*$", text, flags=re.M):
        out[name] = int(val)
    return out
