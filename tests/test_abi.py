"""The C-ABI library loads and exports every symbol include/tw_gb300.h declares
(no compute calls: this runs without a GPU)."""
import ctypes
import re
import subprocess

import numpy as np

import pytest

from conftest import ROOT

HEADER = ROOT / "include" / "tw_gb300.h"


def declared_symbols():
    text = HEADER.read_text()
    return sorted(set(re.findall(r"^TW_API\s+(?:const\s+char\*|int|double)\s+(tw_\w+)\s*\(", text, re.M)))


@pytest.fixture(scope="module")
def libpath():
    import tetwild_gb300 as tw
    from tetwild_gb300 import build as twbuild

    if not tw.library_path().exists():
        twbuild.build()
    return tw.library_path()


def test_header_declares_api():
    syms = declared_symbols()
    assert len(syms) >= 20
    assert "tw_amips_soa" in syms and "tw_envelope_points" in syms and "tw_newton_stars" in syms


def test_library_exports_every_declared_symbol(libpath):
    lib = ctypes.CDLL(str(libpath))
    missing = [s for s in declared_symbols() if not hasattr(lib, s)]
    assert not missing, missing


def test_library_exports_nothing_else(libpath):
    out = subprocess.run(["nm", "-D", "--defined-only", str(libpath)], capture_output=True,
                         text=True, check=True).stdout
    exported = sorted({l.split()[-1] for l in out.splitlines() if " T " in l and l.split()[-1].startswith("tw_")})
    assert exported == declared_symbols()


def test_python_binding_covers_header():
    import tetwild_gb300 as tw

    assert sorted(tw.EXPORTED_SYMBOLS) == declared_symbols()


def test_python_binding_loads(libpath):
    import tetwild_gb300 as tw

    lib = tw.load_library()
    assert lib.tw_last_error(None) == b"null context"
    assert lib.tw_ctx_destroy(None) == tw.TW_ERR_ARG


def test_no_cpu_fallback_without_library(tmp_path, monkeypatch):
    import tetwild_gb300 as tw

    monkeypatch.setattr(tw, "_LIB", None)
    monkeypatch.setattr(tw, "library_path", lambda: tmp_path / "missing.so")
    with pytest.raises(tw.TetWildGpuError):
        tw.Context(0)


def test_synthetic_shapes():
    from tetwild_gb300 import synthetic as syn

    V, F = syn.displaced_sphere(seed=0)
    assert F.shape == (100000, 3) and V.shape == (50002, 3)
    V, F = syn.icosphere(3)
    assert V.shape == (642, 3) and F.shape == (1280, 3)
    T = syn.energy_batch(1000, seed=0)
    assert T.shape == (12, 1000)
    xyz, off, tets, cen = syn.star_batch(20, seed=0)
    n = off[1:] - off[:-1]
    assert n.min() >= 4 and n.max() <= 96 and len(cen) == 20


def test_filter_energy_rule_matches_oracle(oracle):
    """tw_filter_energy is host code: its choice over bucket histograms equals
    the oracle's restatement of getFilterEnergy (LocalOperations.cpp:674-692)."""
    import tetwild_gb300 as tw

    rng = np.random.default_rng(0)
    lib = tw.load_library()
    for _ in range(2000):
        b = np.zeros(11, np.int64)
        k = rng.integers(1, 11)
        b[rng.choice(11, k, replace=False)] = rng.integers(0, 50, k)
        for thres in (10.0, 8.0):
            c = ctypes.c_int()
            e = lib.tw_filter_energy(b.ctypes.data, thres, ctypes.byref(c))
            assert (e, bool(c.value)) == oracle.filter_energy(b, thres)


def _header_signatures():
    """{name: (return kind, [parameter kinds])} from the TW_API declarations; a kind is
    'p' (pointer), 'f8' (double), 'f4' (float) or 'iN' (an integer of N bytes)."""
    text = re.sub(r"/\*.*?\*/", " ", HEADER.read_text(), flags=re.S)
    ints = {"int": 4, "int32_t": 4, "uint32_t": 4, "int64_t": 8, "uint64_t": 8, "size_t": 8,
            "uint8_t": 1, "char": 1}

    def kind(decl):
        decl = decl.strip()
        if "*" in decl:
            return "p"
        words = [w for w in re.findall(r"\w+", decl) if w not in ("const", "unsigned")]
        if words[0] == "double":
            return "f8"
        if words[0] == "float":
            return "f4"
        return f"i{ints[words[0]]}"

    sigs = {}
    for m in re.finditer(r"^TW_API\s+([^(]*?)\s*\b(tw_\w+)\s*\(([^)]*)\)\s*;", text, re.M):
        ret, name, params = m.groups()
        ps = [q for q in params.split(",") if q.strip() and q.strip() != "void"]
        sigs[name] = ("p" if "*" in ret else kind(ret), [kind(q) for q in ps])
    return sigs


def _ctypes_kind(t):
    if t is ctypes.c_void_p or t is ctypes.c_char_p or hasattr(t, "_type_") and \
            isinstance(getattr(t, "_type_"), type):
        return "p"
    if t in (ctypes.c_double,):
        return "f8"
    if t in (ctypes.c_float,):
        return "f4"
    return f"i{ctypes.sizeof(t)}"


def test_python_signatures_match_header():
    """Every ctypes argument list (and return type) in the Python binding has the
    parameter count, pointer-ness and integer/float widths of the header's
    declaration, so no call passes a 4-byte int where the C side reads 8 bytes."""
    import tetwild_gb300 as tw

    sigs = _header_signatures()
    assert sorted(sigs) == declared_symbols()
    bad = []
    for name, args in tw._SIGS.items():
        ret, params = sigs[name]
        got = [_ctypes_kind(a) for a in args]
        if got != params:
            bad.append((name, got, params))
        want_ret = ("p" if name.endswith("last_error") else
                    "f8" if name == "tw_filter_energy" else "i4")
        if ret != want_ret:
            bad.append((name, "return", ret, want_ret))
    assert not bad, bad


@pytest.mark.parametrize("compiler,std,ext", [("gcc", "-std=c99", "c"), ("g++", "-std=c++17", "cpp")])
def test_header_compiles_for_c_and_cpp_hosts(tmp_path, compiler, std, ext):
    """The header is valid C99 and C++17 on its own (a C, C++ or cgo host includes it as
    is), and every declared symbol is a function with C linkage of that name."""
    import shutil

    if shutil.which(compiler) is None:
        pytest.skip(f"{compiler} not installed")
    syms = declared_symbols()
    src = tmp_path / f"use_header.{ext}"
    src.write_text('#include "tw_gb300.h"\n'
                   "typedef void (*fn)(void);\n"
                   "fn const table[] = {\n" +
                   "".join(f"    (fn)&{s},\n" for s in syms) + "};\n")
    r = subprocess.run([compiler, std, "-Wall", "-Wextra", "-Werror", "-pedantic",
                        "-I", str(HEADER.parent), "-c", str(src), "-o", str(tmp_path / "u.o")],
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    out = subprocess.run(["nm", "-u", str(tmp_path / "u.o")], capture_output=True, text=True,
                         check=True).stdout
    assert sorted(l.split()[-1] for l in out.splitlines() if "tw_" in l) == syms


def test_python_constants_match_the_header():
    """Every integer #define of the header that the binding mirrors (TW_* module
    constants, Context.TUNE_* knobs) has the header's value."""
    import tetwild_gb300 as tw

    defines = {m.group(1): int(m.group(2)) for m in
               re.finditer(r"^#define\s+(TW_\w+)\s+\(?(-?\d+)\)?\s*(?:/\*.*)?$", HEADER.read_text(), re.M)}
    assert defines, "no integer defines parsed"
    checked = 0
    for name, value in defines.items():
        if name.startswith("TW_TUNE_"):
            attr = name[len("TW_"):]
            assert getattr(tw.Context, attr) == value, name
            checked += 1
        elif hasattr(tw, name):
            assert getattr(tw, name) == value, name
            checked += 1
    assert checked >= 45, checked
