"""The Rust binding a maintainer adds to the reference crate
(integration/rust/src/gi/ffi.rs and the GiStage in mod.rs) cannot be compiled
in this image (no cargo).  This checks it against the C header without Rust:
every `#[repr(C)]` struct's size and field offsets, computed with C layout
rules from the Rust field types, must equal what gcc reports for the same
struct of `include/rc.h`; every `extern "C"` function must be declared in the
header with the same number of parameters, and every function of the header
must be bound."""
import os
import re
import subprocess

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
FFI = os.path.join(ROOT, "integration", "rust", "src", "gi", "ffi.rs")
STAGE = os.path.join(ROOT, "integration", "rust", "src", "gi", "mod.rs")
HDR = os.path.join(ROOT, "include", "rc.h")
SCALARS = {"i8": 1, "u8": 1, "i16": 2, "u16": 2, "i32": 4, "u32": 4, "f32": 4, "i64": 8, "u64": 8, "f64": 8,
           "c_int": 4, "c_char": 1}


def _rust_block():
    text = open(FFI).read()
    return re.sub(r"//[^\n]*", "", text)


def _header_functions():
    hdr = re.sub(r"/\*.*?\*/", "", open(HDR).read(), flags=re.S)
    return hdr, set(re.findall(r"\b(rc_\w+)\s*\([^)]*\)\s*;", hdr))


def _rust_structs(block):
    out = {}
    for name, body in re.findall(r"#\[repr\(C\)\](?:\s*#\[[^\]]*\])*\s*pub struct (\w+)\s*\{(.*?)\}", block, re.S):
        fields = re.findall(r"(?:pub\s+)?(\w+)\s*:\s*([^,]+?)\s*(?:,|$)", body.strip())
        out[name] = [(f, t.strip()) for f, t in fields]
    return out


def _consts():
    """usize constants of the binding (array lengths)."""
    return {k: int(v) for k, v in re.findall(r"pub const (\w+): usize = (\d+);", _rust_block())}


def _layout(ty, structs, memo):
    """(size, align) of a Rust field type under C layout rules."""
    ty = ty.strip()
    m = re.fullmatch(r"\[(.+);\s*(\w+)\]", ty)
    if m:
        s, a = _layout(m.group(1), structs, memo)
        count = m.group(2)
        return s * (int(count) if count.isdigit() else _consts()[count]), a
    if ty.startswith("*"):
        return 8, 8
    if ty in SCALARS:
        return SCALARS[ty], SCALARS[ty]
    return _struct_layout(ty, structs, memo)[:2]


def _struct_layout(name, structs, memo):
    if name in memo:
        return memo[name]
    off, align, offsets = 0, 1, {}
    for f, t in structs[name]:
        s, a = _layout(t, structs, memo)
        off = (off + a - 1) // a * a
        offsets[f] = off
        off += s
        align = max(align, a)
    size = (off + align - 1) // align * align
    memo[name] = (size, align, offsets)
    return memo[name]


def _c_layouts(structs, tmp_path):
    lines = ['#include <stddef.h>', '#include <stdio.h>', '#include "rc.h"', "int main(void) {"]
    for name, fields in structs.items():
        lines.append('  printf("%s size %%zu\\n", sizeof(%s));' % (name, name))
        for f, _ in fields:
            if f.startswith("_"):
                continue
            lines.append('  printf("%s.%s %%zu\\n", offsetof(%s, %s));' % (name, f, name, f))
    lines.append("  return 0;\n}")
    src = tmp_path / "layout.c"
    src.write_text("\n".join(lines))
    exe = tmp_path / "layout"
    subprocess.run(["gcc", "-std=c11", "-I", os.path.dirname(HDR), str(src), "-o", str(exe)], check=True)
    out = {}
    for line in subprocess.run([str(exe)], check=True, capture_output=True, text=True).stdout.splitlines():
        k, v = line.rsplit(" ", 1)
        out[k] = int(v)
    return out


def test_rust_structs_match_the_c_layout(tmp_path):
    structs = {k: v for k, v in _rust_structs(_rust_block()).items() if not all(f.startswith("_") for f, _ in v)}
    assert {"rc_params", "rc_voxel", "rc_box", "rc_sphere", "rc_scene_spec", "rc_level_info", "rc_batch_tiles",
            "rc_nrc_params", "rc_nrc_stats", "rc_shade_material", "rc_texture", "rc_shade_view"} <= set(structs)
    c = _c_layouts(structs, tmp_path)
    memo = {}
    for name in structs:
        size, _, offsets = _struct_layout(name, structs, memo)
        assert size == c["%s size" % name], name
        for f, off in offsets.items():
            assert off == c["%s.%s" % (name, f)], (name, f)


def test_rust_functions_are_declared_in_the_header():
    block = _rust_block()
    fns = re.findall(r"pub fn (\w+)\((.*?)\)\s*(?:->\s*[^;]+)?;", block, re.S)
    hdr, declared = _header_functions()
    assert declared == {name for name, _ in fns}, declared ^ {name for name, _ in fns}
    for name, params in fns:
        m = re.search(r"\b%s\s*\(([^)]*)\)\s*;" % name, hdr, re.S)
        assert m, "%s is not declared in include/rc.h" % name
        cp = m.group(1).strip()
        n_c = 0 if cp in ("", "void") else cp.count(",") + 1
        n_r = 0 if not params.strip() else params.count(",") + 1
        assert n_c == n_r, (name, n_c, n_r)


def test_stage_implements_the_render_stage_trait():
    """GiStage provides the three methods of RenderStage<T> (reference:
    src/app.rs:3-7) and calls only functions the binding declares."""
    text = open(STAGE).read()
    assert re.search(r"impl RenderStage<AppState> for GiStage", text)
    for method in ("update", "render", "resize"):
        assert re.search(r"fn %s\(" % method, text), method
    bound = set(re.findall(r"pub fn (\w+)\(", _rust_block()))
    used = set(re.findall(r"\b(rc_\w+)\(", text))
    assert used and used <= bound, used - bound
