"""The Rust binding (rust/vonkarman-gpu-sys/src/lib.rs) against the C header
(include/vonkarman_gpu.h), on the CPU and without a Rust toolchain: the
extern block declares every entry point of the header with the same argument
count and argument / return types, the #[repr(C)] structs vk_config and
vk_tier1_out list the header's fields in the header's order with the same
types, and the constants carry the header's values."""

import os
import re

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HEADER = os.path.join(ROOT, "include", "vonkarman_gpu.h")
SYS = os.path.join(ROOT, "rust", "vonkarman-gpu-sys", "src", "lib.rs")
SAFE = os.path.join(ROOT, "rust", "vonkarman-gpu", "src", "lib.rs")

C2RUST = {"int": "c_int", "int32_t": "i32", "int64_t": "i64", "uint64_t": "u64", "double": "f64",
          "size_t": "usize", "void": "c_void", "char": "c_char", "vk_ctx": "vk_ctx", "vk_fft": "vk_fft",
          "vk_config": "vk_config", "vk_tier1_out": "vk_tier1_out"}


def header_src():
    return re.sub(r"/\*.*?\*/", "", open(HEADER).read(), flags=re.S)


def c_type_to_rust(t: str) -> str:
    t = t.strip()
    const = t.startswith("const ")
    if const:
        t = t[6:].strip()
    stars = t.count("*")
    base = C2RUST[t.replace("*", "").strip()]
    out = base
    for i in range(stars):
        out = ("*const " if const and i == 0 else "*mut ") + out
    return out


def header_functions():
    out = {}
    for ret, name, args in re.findall(r"^\s*((?:const\s+)?[a-z_0-9]+\s*\**)\s*(vk_[a-z0-9_]+)\s*\(([^)]*)\)\s*;",
                                      header_src(), flags=re.M):
        types = []
        args = args.strip()
        if args and args != "void":
            for a in args.split(","):
                m = re.match(r"(.*?)([A-Za-z_][A-Za-z_0-9]*)$", a.strip())
                types.append(c_type_to_rust(m.group(1)))
        r = c_type_to_rust(ret)
        out[name] = (types, None if r == "c_void" else r)
    return out


def rust_functions():
    src = open(SYS).read()
    block = src[src.index('unsafe extern "C" {'):]
    out = {}
    for name, args, ret in re.findall(r"pub fn (vk_[a-z0-9_]+)\(([^)]*)\)\s*(?:->\s*([^;]+))?;", block):
        types = [a.split(":", 1)[1].strip() for a in args.split(",") if a.strip()]
        out[name] = (types, ret.strip() if ret else None)
    return out


def test_extern_block_mirrors_every_header_function():
    h, r = header_functions(), rust_functions()
    assert len(h) >= 45
    assert sorted(h) == sorted(r), (set(h) ^ set(r))
    for name in h:
        assert h[name][0] == r[name][0], (name, h[name][0], r[name][0])
        assert h[name][1] == r[name][1], (name, h[name][1], r[name][1])


def _c_struct(name):
    body = re.search(r"typedef struct %s \{(.*?)\}" % name, header_src(), flags=re.S).group(1)
    fields = []
    for decl in body.split(";"):
        decl = decl.strip()
        if not decl:
            continue
        t, names = decl.split(None, 1)
        for nm in names.split(","):
            fields.append((nm.strip(), C2RUST[t]))
    return fields


def _rust_struct(name):
    src = open(SYS).read()
    body = re.search(r"pub struct %s \{(.*?)\}" % name, src, flags=re.S).group(1)
    return [(m.group(1), m.group(2)) for m in re.finditer(r"pub (\w+): (\w+),", body)]


def test_repr_c_structs_match_header_field_order():
    for name in ("vk_config", "vk_tier1_out"):
        assert _c_struct(name) == _rust_struct(name), name
    src = open(SYS).read()
    for name in ("vk_config", "vk_tier1_out"):
        assert re.search(r"#\[repr\(C\)\]\s*#\[derive\([^)]*\)\]\s*pub struct %s" % name, src), name


def test_constants_match_header():
    hs = header_src()
    want = {m.group(1): int(m.group(2)) for m in re.finditer(r"\b(VK_[A-Z0-9_]+)\s*=\s*(\d+)", hs)}
    want.update({m.group(1): int(m.group(2)) for m in re.finditer(r"#define (VK_[A-Z0-9_]+) (\d+)", hs)})
    got = {m.group(1): int(m.group(2)) for m in re.finditer(r"pub const (VK_[A-Z0-9_]+): \w+ = (\d+);",
                                                              open(SYS).read())}
    assert set(want) <= set(got), set(want) - set(got)
    for k, v in want.items():
        assert got[k] == v, k


def test_safe_crate_implements_the_reference_traits():
    src = open(SAFE).read()
    assert "impl FftBackend<f64> for NativeGpuBackend" in src
    assert "impl Domain<f64> for Periodic3DGpu" in src
    # every Domain method (vonkarman-core/src/domain.rs:39-81) is implemented
    for m in ("step", "time", "step_count", "dt", "energy", "enstrophy", "helicity", "superhelicity",
              "max_vorticity", "cfl_dt", "u_hat", "grid", "params", "snapshot"):
        assert re.search(r"fn %s\(&" % m, src), m
    for m in ("r2c_3d", "c2r_3d", "name", "precision_digits"):
        assert re.search(r"fn %s\(&self" % m, src), m
    # every sys call the safe crate makes exists in the binding
    used = set(re.findall(r"sys::(vk_[a-z0-9_]+)\(", src))
    assert used <= set(rust_functions()), used - set(rust_functions())
