"""The Rust FFI crate (rust/ferrolearn-cluster-cuda, which cannot be compiled
here: no cargo) against the C ABI it binds: every struct of
include/ferrokmeans.h must appear in src/ffi.rs with the same fields in the
same order and matching types, and every function with the same parameters
and return type, so that the crate's #[repr(C)] layouts and calls are the
library's."""
import os
import re

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HEADER = os.path.join(ROOT, "include", "ferrokmeans.h")
FFI = os.path.join(ROOT, "rust", "ferrolearn-cluster-cuda", "src", "ffi.rs")

_SCALAR = {"int64_t": "i64", "uint64_t": "u64", "int32_t": "i32", "double": "f64", "float": "f32",
           "uint16_t": "u16", "char": "c_char", "void": "c_void", "fk_ctx": "fk_ctx", "fk_status": "i32",
           "fk_kmeans_params": "fk_kmeans_params", "fk_fit_report": "fk_fit_report",
           "fk_batch_problem": "fk_batch_problem", "fk_batch_report": "fk_batch_report",
           "fk_minibatch_params": "fk_minibatch_params", "fk_bisecting_params": "fk_bisecting_params"}


def _strip_c_comments(s):
    return re.sub(r"/\*.*?\*/", " ", s, flags=re.S)


def _c_type(decl):
    """'const double *x' -> ('x', '*const f64'); 'int32_t v[20]' -> ('v', '[i32; 20]')."""
    decl = decl.strip()
    m = re.match(r"^(.*?)([A-Za-z_]\w*)\s*(\[(\d+)\])?$", decl)
    base, name, arr = m.group(1).strip(), m.group(2), m.group(4)
    const = base.startswith("const ")
    base = base.replace("const ", "").strip()
    stars = base.count("*")
    base = base.replace("*", "").strip()
    t = _SCALAR[base]
    if stars:
        t = ("*const " if const else "*mut ") + t
        for _ in range(stars - 1):
            t = "*mut " + t
    if arr:
        t = f"[{t}; {arr}]"
    return name, t


def header_structs():
    src = _strip_c_comments(open(HEADER).read())
    out = {}
    for m in re.finditer(r"typedef struct (\w+) \{(.*?)\} \1;", src, flags=re.S):
        fields = []
        for stmt in m.group(2).split(";"):
            stmt = " ".join(stmt.split())
            if not stmt:
                continue
            first, *rest = [p.strip() for p in stmt.split(",")]
            mm = re.match(r"^(.*?)([A-Za-z_]\w*\s*(\[\d+\])?)$", first)
            base = mm.group(1)
            for decl in [mm.group(2)] + rest:
                fields.append(_c_type(base + " " + decl))
        out[m.group(1)] = fields
    return out


def header_functions():
    src = _strip_c_comments(open(HEADER).read())
    out = {}
    for m in re.finditer(r"(fk_status|void|uint64_t|const char \*)\s*(fk_\w+)\(([^)]*)\);", src):
        ret = {"fk_status": "i32", "void": None, "uint64_t": "u64", "const char *": "*const c_char"}[m.group(1)]
        args = [" ".join(a.split()) for a in m.group(3).split(",")]
        params = [] if args == ["void"] else [_c_type(a)[1] for a in args]
        out[m.group(2)] = (params, ret)
    return out


def rust_structs():
    src = open(FFI).read()
    out = {}
    for m in re.finditer(r"pub struct (\w+) \{(.*?)\n\}", src, flags=re.S):
        fields = re.findall(r"pub (\w+): ([^,\n]+),", m.group(2))
        out[m.group(1)] = [(n, " ".join(t.split())) for n, t in fields]
    return out


def rust_functions():
    src = open(FFI).read()
    block = src[src.index('unsafe extern "C" {'):]
    out = {}
    for m in re.finditer(r"pub fn (\w+)\((.*?)\)\s*(->\s*([^;]+))?;", block, flags=re.S):
        args = [a.strip() for a in " ".join(m.group(2).split()).split(",") if a.strip()]
        params = [a.split(":", 1)[1].strip() for a in args]
        ret = m.group(4).strip() if m.group(4) else None
        out[m.group(1)] = (params, ret)
    return out


def test_every_struct_matches_the_header():
    hs, rs = header_structs(), rust_structs()
    assert set(hs) == {"fk_kmeans_params", "fk_fit_report", "fk_batch_problem", "fk_batch_report",
                       "fk_minibatch_params", "fk_bisecting_params"}
    for name, fields in hs.items():
        assert name in rs, name
        assert rs[name] == fields, (name, rs[name], fields)


def test_every_function_matches_the_header():
    hf, rf = header_functions(), rust_functions()
    assert len(hf) >= 30
    assert set(hf) == set(rf), (set(hf) ^ set(rf))
    for name, sig in hf.items():
        assert rf[name] == sig, (name, rf[name], sig)


def test_status_and_enum_constants_match_the_header():
    src = _strip_c_comments(open(HEADER).read())
    consts = dict(re.findall(r"\b(FK_[A-Z0-9_]+) = (\d+)", src))
    rust = dict(re.findall(r"pub const (FK_[A-Z0-9_]+): i32 = (\d+);", open(FFI).read()))
    assert consts == rust
