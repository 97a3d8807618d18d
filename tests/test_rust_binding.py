"""The Rust binding (rust/feriphys-gb300-sys) declares exactly the C ABI of
include/feriphys_gb300.h: every function, with the same parameter names,
order and types, and the same #[repr(C)] struct layouts.  No Rust toolchain
exists in this image, so the binding is checked here by reading both files;
the safe wrapper crate (rust/feriphys-gb300) may only call declared functions.
"""
import os
import re

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HEADER = os.path.join(ROOT, "include", "feriphys_gb300.h")
SYS = os.path.join(ROOT, "rust", "feriphys-gb300-sys", "src", "lib.rs")
SAFE = os.path.join(ROOT, "rust", "feriphys-gb300", "src", "lib.rs")

# C parameter type -> the Rust type the binding must use
C_TO_RUST = {
    "const fgb_config*": "*const FgbConfig", "fgb_config*": "*mut FgbConfig",
    "const fgb_mesh*": "*const FgbMesh", "fgb_mesh*": "*mut FgbMesh", "fgb_mesh* const*": "*const *mut FgbMesh",
    "fgb_mesh**": "*mut *mut FgbMesh", "const fgb_obstacle*": "*const FgbObstacle", "fgb_obstacle*": "*mut FgbObstacle",
    "fgb_obstacle* const*": "*const *mut FgbObstacle", "fgb_obstacle**": "*mut *mut FgbObstacle",
    "const fgb_sim*": "*const FgbSim", "fgb_sim*": "*mut FgbSim", "fgb_sim**": "*mut *mut FgbSim",
    "const fgb_spring_override*": "*const FgbSpringOverride", "const fgb_surrogate*": "*const FgbSurrogate",
    "fgb_surrogate*": "*mut FgbSurrogate", "fgb_surrogate**": "*mut *mut FgbSurrogate",
    "const fgb_surrogate_check*": "*const FgbSurrogateCheck", "const float[]": "*const f32",
    "const float*": "*const f32", "const uint32_t*": "*const u32", "double*": "*mut f64", "float": "f32",
    "float*": "*mut f32", "int": "c_int", "int*": "*mut c_int", "int32_t": "i32", "int64_t[]": "*mut i64",
    "uint32_t": "u32", "uint32_t*": "*mut u32", "uint64_t": "u64", "uint64_t[]": "*mut u64",
    "uint64_t*": "*mut u64", "void*": "*mut c_void", "const char*": "*const c_char",
}
RUST_KEYWORDS = {"in": "input"}
C_FIELD = {"int32_t": "i32", "float": "f32", "uint32_t": "u32"}


def header_functions():
    s = re.sub(r"/\*.*?\*/", "", open(HEADER).read(), flags=re.S)
    out = {}
    for ret, name, args in re.findall(r"\n([A-Za-z_][\w\s\*]*?)\b(fgb_\w+)\s*\(([^;{]*?)\)\s*;", s):
        params = []
        for a in args.split(","):
            a = " ".join(a.split())
            if a in ("", "void"):
                continue
            m = re.match(r"(.*?)\b(\w+)\s*(\[\d*\])?$", a)
            ctype = m.group(1).strip() + ("[]" if m.group(3) else "")
            pname = RUST_KEYWORDS.get(m.group(2), m.group(2))
            params.append((pname, C_TO_RUST[ctype]))
        out[name] = (params, C_TO_RUST[ret.strip()])
    return out


def rust_functions():
    s = open(SYS).read()
    block = s[s.index('extern "C" {'):]
    block = re.sub(r"//[^\n]*", "", block)
    out = {}
    for name, args, ret in re.findall(r"pub fn (fgb_\w+)\s*\(([^)]*)\)\s*(?:->\s*([^;]+))?;", block, re.S):
        params = []
        for a in args.split(","):
            a = " ".join(a.split())
            if not a:
                continue
            pname, ptype = a.split(":", 1)
            params.append((pname.strip(), ptype.strip()))
        out[name] = (params, ret.strip() if ret else "")
    return out


def struct_fields(text, name, rust):
    if rust:
        m = re.search(r"pub struct %s \{(.*?)\}" % name, text, re.S)
        return [tuple(x) for x in re.findall(r"pub (\w+): ([^,]+),", m.group(1))]
    m = re.search(r"typedef struct %s \{(.*?)\} %s;" % (name, name), re.sub(r"/\*.*?\*/", "", text, flags=re.S), re.S)
    fields = []
    for line in m.group(1).split(";"):
        line = " ".join(line.split())
        if not line:
            continue
        ctype, names = line.split(" ", 1)
        for nm in names.split(","):
            nm = nm.strip()
            arr = re.match(r"(\w+)\[(\d+)\]", nm)
            if arr:
                fields.append((arr.group(1), "[%s; %s]" % (C_FIELD[ctype], arr.group(2))))
            else:
                fields.append((nm, C_FIELD[ctype]))
    return fields


def test_every_entry_point_declared_with_the_same_signature():
    h, r = header_functions(), rust_functions()
    assert len(h) >= 60
    assert sorted(h) == sorted(r), (set(h) ^ set(r))
    for name, (params, ret) in h.items():
        assert r[name] == (params, ret), (name, r[name], (params, ret))


def test_declared_in_header_order():
    h = list(header_functions())
    r = list(rust_functions())
    assert h == r


def test_repr_c_structs_match_the_header():
    hs, rs = open(HEADER).read(), open(SYS).read()
    for c_name, r_name in (("fgb_config", "FgbConfig"), ("fgb_spring_override", "FgbSpringOverride"),
                           ("fgb_surrogate_check", "FgbSurrogateCheck")):
        assert struct_fields(hs, c_name, False) == struct_fields(rs, r_name, True), c_name
        assert re.search(r"#\[repr\(C\)\][^\n]*\n(#\[derive[^\n]*\n)?pub struct %s \{" % r_name, rs), r_name


def test_status_codes_match_the_header():
    hs, rs = open(HEADER).read(), open(SYS).read()
    status = hs[hs.index("typedef enum fgb_status"):hs.index("} fgb_status;")]
    codes = re.findall(r"(FGB_\w+) = (-?\d+)", status)
    assert len(codes) == 8
    for name, val in codes:
        assert re.search(r"pub const %s: c_int = %s;" % (name, val), rs), name
    for name, val in re.findall(r"(FGB_EULER|FGB_RK4) = (\d+)", hs):
        assert re.search(r"pub const %s: i32 = %s;" % (name, val), rs), name


def test_safe_wrappers_call_declared_functions_only():
    declared = set(rust_functions())
    used = set(re.findall(r"sys::(fgb_\w+)", open(SAFE).read()))
    assert used and used <= declared, used - declared
