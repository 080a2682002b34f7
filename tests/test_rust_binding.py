"""The Rust binding (rust/bioshell-crmsd-sys/src/lib.rs) against the C header
(include/bioshell_crmsd.h), checked mechanically on the CPU: no Rust
toolchain is needed.

* every exported function of the header has one `extern "C"` declaration
  with the same parameter and return types (C types mapped to their Rust
  equivalents), and the binding declares nothing the header does not;
* every struct of the header has a `#[repr(C)]` mirror with the same fields
  in the same order and of the same types, and every opaque handle a
  zero-sized `#[repr(C)]` type;
* every integer constant of the header has a `pub const` of the same value;
* the safe API (rust/bioshell-pdb/src/calc/crmsd.rs) and the clustering
  impls call only functions the binding declares.
A field added to a header struct, or a changed signature, fails here."""
import os
import re

import pytest

import c_header as H

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
SYS = os.path.join(ROOT, "rust", "bioshell-crmsd-sys", "src", "lib.rs")
SAFE = os.path.join(ROOT, "rust", "bioshell-pdb", "src", "calc", "crmsd.rs")
POINTS = os.path.join(ROOT, "rust", "bioshell-clustering", "src", "crmsd_points.rs")

SCALARS = {"int32_t": "i32", "int64_t": "i64", "uint32_t": "u32", "size_t": "usize", "double": "f64",
           "float": "f32", "char": "c_char", "void": "c_void", "bs_status": "BsStatus"}
NAMED = {"bs_ctx": "BsCtx", "bs_server": "BsServer", "bs_models": "BsModels", "bs_tsv": "BsTsv",
         "bs_opts": "BsOpts", "bs_metrics": "BsMetrics", "bs_set_desc": "BsSetDesc",
         "bs_server_config": "BsServerConfig", "bs_server_stats": "BsServerStats"}


def rust_type(c: str) -> str:
    """'const double *const *' -> '*const *const f64'; 'int32_t[6]' -> '[i32; 6]'."""
    c = c.strip()
    m = re.match(r"^(.*)\[(\d+)\]$", c)
    if m:
        return f"[{rust_type(m.group(1))}; {m.group(2)}]"
    if c == "void":
        return "()"
    # peel pointer levels from the right: "T *", "T *const *"
    if c.endswith("*"):
        inner = c[:-1].rstrip()
        const_ptr = False
        if inner.endswith("*const"):  # "... *const" is a const pointer level
            inner, const_ptr = inner[:-len("const")].rstrip(), True
        if inner.endswith("*"):
            pointee = rust_type(inner)
            return ("*const " if const_ptr else "*mut ") + pointee
        const = inner.startswith("const ")
        base = inner[len("const "):] if const else inner
        return ("*const " if const else "*mut ") + ("c_void" if base == "void" else rust_type(base))
    return SCALARS.get(c) or NAMED[c]


def _norm_rs(t: str) -> str:
    t = re.sub(r"\s+", " ", t.strip())
    return t.replace("* const", "*const").replace("* mut", "*mut")


def rust_functions():
    text = re.sub(r"//[^\n]*", "", open(SYS).read())
    block = text[text.index('extern "C" {'):]
    out = {}
    for m in re.finditer(r"pub fn (\w+)\s*\(([^)]*)\)\s*(->\s*([^;]+))?;", block, flags=re.S):
        params = [p for p in m.group(2).split(",") if p.strip()]
        types = [_norm_rs(p.split(":", 1)[1]) for p in params]
        out[m.group(1)] = (_norm_rs(m.group(4)) if m.group(4) else "()", types)
    return out


def rust_structs():
    text = re.sub(r"//[^\n]*", "", open(SYS).read())
    out = {}
    for m in re.finditer(r"#\[repr\(C\)\]\s*(?:#\[derive\([^)]*\)\]\s*)?pub struct (\w+)\s*\{(.*?)\}", text, flags=re.S):
        fields = []
        for f in m.group(2).split(","):
            f = f.strip()
            if not f:
                continue
            name, typ = f.split(":", 1)
            fields.append((name.replace("pub ", "").strip(), _norm_rs(typ)))
        out[m.group(1)] = fields
    return out


def rust_consts():
    text = open(SYS).read()
    return {k: int(v) for k, v in re.findall(r"pub const (BS_\w+): i32 = (-?\d+);", text)}


def test_type_mapping():
    assert rust_type("const double *") == "*const f64"
    assert rust_type("bs_ctx **") == "*mut *mut BsCtx"
    assert rust_type("const char *const *") == "*const *const c_char"
    assert rust_type("const double *const *") == "*const *const f64"
    assert rust_type("void *") == "*mut c_void"
    assert rust_type("int32_t[6]") == "[i32; 6]"
    assert rust_type("void") == "()"


def test_every_header_function_is_bound_with_the_same_types():
    c = H.functions()
    r = rust_functions()
    assert set(c) == set(r), f"header only: {sorted(set(c) - set(r))}; binding only: {sorted(set(r) - set(c))}"
    for name, (ret, params) in c.items():
        rret, rparams = r[name]
        want_ret = "()" if ret == "void" else rust_type(ret)
        assert rret == want_ret, f"{name}: returns {rret}, header {ret}"
        assert len(rparams) == len(params), f"{name}: {len(rparams)} parameters, header {len(params)}"
        for k, (rp, cp) in enumerate(zip(rparams, params)):
            assert rp == rust_type(cp), f"{name} parameter {k}: {rp}, header {cp}"


def test_structs_mirror_the_header():
    cs = H.structs()
    rs = rust_structs()
    for cname, fields in cs.items():
        rname = NAMED[cname]
        assert rname in rs, f"no #[repr(C)] mirror of {cname}"
        rf = rs[rname]
        assert [n.lower() for n, _ in fields] == [n for n, _ in rf], f"{cname}: field names or order differ"
        for (n, ct), (_, rt) in zip(fields, rf):
            assert rt == rust_type(ct), f"{cname}.{n}: {rt}, header {ct}"
    for opaque in H.opaque_types():
        assert rs.get(NAMED[opaque]) == [("_p", "[u8; 0]")], f"opaque {opaque} is not a zero-sized repr(C) type"


def test_constants_match():
    c = H.constants()
    r = rust_consts()
    for k, v in c.items():
        assert r.get(k) == v, f"{k}: binding {r.get(k)}, header {v}"


def test_safe_code_calls_only_bound_functions():
    declared = set(rust_functions())
    used = set(re.findall(r"\b(bs_\w+)\s*\(", open(SAFE).read()))
    assert used and used <= declared, sorted(used - declared)
    # the clustering impls use the safe API's public types only
    safe = open(SAFE).read()
    imported = re.findall(r"use bioshell_pdb::calc::\{([^}]*)\}", open(POINTS).read())
    names = [n.strip() for n in imported[0].split(",")]
    for n in names:
        assert re.search(rf"pub struct {n}\b", safe), n


def test_safe_api_surface():
    text = open(SAFE).read()
    for sig in ("pub fn crmsd<T: HasCartesians>(a: &[T], b: &[T]) -> Result<f64, PDBError>",
                "pub fn crmsd_all_vs_all<T: HasCartesians>(models: &[&[T]], opts: &CrmsdOptions)",
                "pub fn crmsd_batched<T: HasCartesians>(sets: &[&[&[T]]], opts: &CrmsdOptions)",
                "pub fn model_coordinates(&self, i: usize) -> &[Vec3]",
                "pub fn as_f32_closure(&self)", "pub struct CrmsdServer", "pub fn cancel(&self, t: &Ticket)"):
        assert sig in text, sig
    pts = open(POINTS).read()
    for impl in ("impl DistanceByIndex for CrmsdPoints", "impl NeighborsOf for CrmsdPoints",
                 "impl DistanceByIndex for CrmsdNeighborPoints", "impl NeighborsOf for CrmsdNeighborPoints"):
        assert impl in pts, impl
