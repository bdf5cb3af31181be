"""The C-ABI library builds, loads without a GPU and exports every function include/rcg.h declares.

No compute call is made here (no GPU on the CPU test runner)."""

import ctypes
import os
import re

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _declared():
    src = open(os.path.join(ROOT, "include", "rcg.h")).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    return sorted(set(re.findall(r"\b(rcg_[a-z0-9_]+)\s*\(", src)))


def _lib():
    import importlib.util
    import sys

    sys.path.insert(0, os.path.join(ROOT, "rust-compress_gb300"))
    import build as b  # rust-compress_gb300/build.py

    b.build()
    return ctypes.CDLL(b.LIB)


def test_header_declares_the_boundary():
    names = _declared()
    for n in ("rcg_ctx_create", "rcg_ssimulacra2", "rcg_build_coefs", "rcg_reconstruct", "rcg_search"):
        assert n in names


def test_library_exports_every_declared_symbol():
    lib = _lib()
    missing = [n for n in _declared() if not hasattr(lib, n)]
    assert not missing, missing


def test_python_bindings_cover_the_header():
    _lib()
    import rcg

    assert set(_declared()) <= set(rcg.EXPORTED) | set(), set(_declared()) - set(rcg.EXPORTED)


def test_context_creation_fails_cleanly_without_a_device():
    # Without a GPU (this runner) rcg_ctx_create must return an error status, not abort.
    import rcg

    try:
        import torch

        if torch.cuda.is_available():
            return
    except Exception:
        pass
    out = ctypes.c_void_p()
    rc = rcg.lib().rcg_ctx_create(0, ctypes.byref(out))
    assert rc != 0 and not out.value


def test_perceptual_defaults_match_the_python_options():
    import rcg

    _lib()
    o = rcg._PerceptualOpts()
    rcg.lib().rcg_perceptual_defaults(ctypes.byref(o))
    d = rcg.PerceptualOptions()
    assert (o.strength, o.gamma, o.w_min, o.w_max, o.radius, bool(o.keep_smaller), bool(o.gradient_fp64),
            bool(o.strength_by_quality)) == \
        (d.strength, d.gamma, d.w_min, d.w_max, d.radius, d.keep_smaller, d.gradient_fp64, d.strength_by_quality)
    # the strength schedule is host arithmetic: checkable without a GPU
    assert [d.strength_for(q) for q in (1, 69, 70, 84, 85, 100)] == [0.35, 0.35, 0.7, 0.7, 1.0, 1.0]
    assert rcg.PerceptualOptions(strength=0.5, strength_by_quality=False).strength_for(90) == 0.5


def _rust_externs():
    src = open(os.path.join(ROOT, "rust-compress_gb300", "rcg-sys", "src", "lib.rs")).read()
    block = src[src.index('extern "C" {'):]
    out = {}
    for m in re.finditer(r"pub fn (rcg_[a-z0-9_]+)\((.*?)\)", block, flags=re.S):
        args = [a for a in m.group(2).split(",") if a.strip()]
        out[m.group(1)] = len(args)
    return out


def _c_arities():
    src = open(os.path.join(ROOT, "include", "rcg.h")).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    return {m.group(1): len([a for a in m.group(2).split(",") if a.strip()])
            for m in re.finditer(r"\b(rcg_[a-z0-9_]+)\s*\(([^;]*?)\)\s*;", src, flags=re.S)}


def test_rust_binding_matches_the_header():
    """rcg-sys (the uncompiled Rust FFI crate a maintainer adds to rust-compress) declares every header function
    with the same number of parameters."""
    rust, c = _rust_externs(), _c_arities()
    assert set(rust) == set(c), (set(c) - set(rust), set(rust) - set(c))
    assert {k: v for k, v in rust.items() if c[k] != v} == {}
