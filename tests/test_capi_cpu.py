"""The C-ABI library loads and exports its header's symbols; host-only calls (no GPU work)."""
import ctypes
import os
import re

import pytest

import gbblas
from gbblas import _lib
import oracle

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HEADER = os.path.join(ROOT, "include", "gbblas.h")


def declared_functions():
    src = open(HEADER).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    return sorted(set(re.findall(r"\b(gb_[a-z0-9_]+)\s*\(", src)))


def test_library_loads():
    assert os.path.exists(gbblas.LIB_PATH)
    assert gbblas.lib().gb_version() == 100


def test_every_declared_symbol_is_exported():
    names = declared_functions()
    assert "gb_gemm_f64" in names and "gb_jmul_f64" in names
    L = gbblas.lib()
    missing = [n for n in names if not hasattr(L, n)]
    assert not missing, missing


def test_every_declared_symbol_has_a_python_signature():
    assert set(declared_functions()) <= set(_lib.SIGNATURES)


def test_julia_front_end_binds_only_declared_symbols():
    """Every `ccall((:gb_..., libgbblas), ...)` target of the Julia front end (including the
    symbols interpolated from `for (T, f) in ((Float64, :gb_...), ...)` loops) is in the header."""
    src = open(os.path.join(ROOT, "jblas.jl_gb300", "julia", "GBBLAS.jl")).read()
    bound = set(re.findall(r":(gb_[a-z0-9_]+)", src))
    assert {"gb_gemm_f64", "gb_kernel_f64", "gb_gemm_semiring_i32", "gb_gemm_f32_host"} <= bound
    assert bound <= set(declared_functions()), sorted(bound - set(declared_functions()))


def test_julia_tuning_struct_matches_header():
    """GBBLAS.TcTuning is passed by pointer to gb_get/set_tc_tuning and gb_autotune_tc: its
    fields are the header's gb_tc_tuning_t fields, in order, all 32-bit."""
    hdr = open(os.path.join(ROOT, "include", "gbblas.h")).read()
    body = re.search(r"typedef struct \{([^}]*)\} gb_tc_tuning_t;", hdr).group(1)
    c_fields = re.findall(r"int32_t\s+(\w+);", body)
    src = open(os.path.join(ROOT, "jblas.jl_gb300", "julia", "GBBLAS.jl")).read()
    jl = re.search(r"struct TcTuning\n(.*?)\nend", src, re.S).group(1)
    jl_fields = re.findall(r"(\w+)::Int32", jl)
    assert c_fields == jl_fields == ["engine", "band", "tma_store", "panels"]


def test_status_strings():
    L = gbblas.lib()
    for code in range(0, -7, -1):
        assert L.gb_status_string(code)
    assert b"unknown" in L.gb_status_string(-99)


@pytest.mark.parametrize("K", [1, 63, 64, 256, 1000, 4096, 8192, 16384, 70000])
@pytest.mark.parametrize("slices", [1, 3, 8, 12])
def test_ozaki_plan_matches_restatement(K, slices):
    got = gbblas.ozaki_plan(512, 384, K, slices)
    ref = oracle.ozaki_plan(K, slices)
    assert got["bits"] == ref["bits"]
    assert got["k_chunk"] == ref["k_chunk"]
    assert got["products"] == ref["products"]
    assert got["groups"] == len(ref["groups"])
    assert got["flops_tensor"] == 2.0 * 512 * 384 * ref["kb_total"] * 64 * ref["products"]


def test_ozaki_plan_rejects_bad_slices():
    L = gbblas.lib()
    p = _lib.OzakiPlan()
    assert L.gb_plan_ozaki(8, 8, 8, 0, ctypes.byref(p)) == _lib.GB_ERR_INVALID_VALUE
    assert L.gb_plan_ozaki(8, 8, 8, 21, ctypes.byref(p)) == _lib.GB_ERR_INVALID_VALUE
    assert L.gb_plan_ozaki(-1, 8, 8, 3, ctypes.byref(p)) == _lib.GB_ERR_INVALID_VALUE


def test_setters():
    L = gbblas.lib()
    assert L.gb_set_wait_limit_ns(0) == 0
    assert L.gb_set_ozaki_tolerance(-1.0) == _lib.GB_ERR_INVALID_VALUE
    assert L.gb_set_ozaki_tolerance(0.0) == 0


@pytest.mark.parametrize("K", [1, 16, 64, 1000, 4100, 8192, 70000, 1 << 19])
@pytest.mark.parametrize("moduli", [1, 2, 3, 8, 15, 16, 17, 20])
def test_ozaki_crt_plan_matches_restatement(K, moduli):
    t = oracle.crt_bits_for(K, moduli)
    if t == 0:
        with pytest.raises(gbblas.GBError):
            gbblas.ozaki_crt_plan(256, 128, K, moduli)
        return
    got = gbblas.ozaki_crt_plan(256, 128, K, moduli)
    assert got["bits"] == t and got["moduli"] == moduli and got["products"] == moduli
    kb = max(1, (K + 63) // 64)
    nch = (kb + 15) // 16
    assert got["k_chunk"] == 64 * ((kb + nch - 1) // nch)
    assert got["flops_tensor"] == 2.0 * 256 * 128 * kb * 64 * moduli


def _crt_blocks_restated(M, N, panels, sms, host):
    """The block rule restated: 256-tile rounds over sms / 2 SM pairs; three panels cut as
    (w, w, e) for host copies or (e, tiles - 3e, 2e) when neither adds a round, else three
    equal panels, else two; four panels as 2 x 2 blocks when there are two tile rows."""
    tm, tn = -(-M // 256), -(-N // 256)
    panels = min(max(panels, 1), 4, tn)
    prow = 2 if panels == 4 and tm >= 2 else 1
    pcol, rtm, pairs = panels // prow, tm // prow, max(sms // 2, 1)
    rounds = lambda c: -(-rtm * c // pairs)   # noqa: E731
    best, w = rounds(tn), None
    if pcol == 3:
        for e in range(1, tn // 5 + 1):
            if host and rounds((tn - e) // 2) + rounds(tn - e - (tn - e) // 2) + rounds(e) == best:
                w = [(tn - e) // 2, tn - e - (tn - e) // 2, e]
                break
        for e in range(1, tn // 5 + 1):
            if w is None and rounds(e) + rounds(tn - 3 * e) + rounds(2 * e) == best:
                w = [e, tn - 3 * e, 2 * e]
                break
        if w is None and sum(rounds(tn * (p + 1) // 3 - tn * p // 3) for p in range(3)) > best:
            pcol = 2
    if w is None:
        w = [tn * (p + 1) // pcol - tn * p // pcol for p in range(pcol)]
    cols, t = [0], 0
    for x in w:
        t += x
        cols.append(min(t * 256, N))
    rows = [min(tm * p // prow * 256, M) for p in range(prow + 1)]
    return {"rows": rows, "cols": cols}


def test_crt_blocks_known_cuts():
    """8192 x 8192 on 152 SMs: three panels of 2, 26 and 4 tiles (1 + 11 + 2 rounds, as one
    launch); a host call with a pinned C: halves and a narrow last panel (6 + 6 + 2); four
    panels: 2 x 2 blocks; 4096 x 4096: three panels fall back to two halves."""
    assert gbblas.crt_blocks(8192, 8192, 3, 152) == {"rows": [0, 8192], "cols": [0, 512, 7168, 8192]}
    assert gbblas.crt_blocks(8192, 8192, 3, 152, True) == {"rows": [0, 8192], "cols": [0, 3584, 7168, 8192]}
    assert gbblas.crt_blocks(8192, 8192, 4, 152) == {"rows": [0, 4096, 8192], "cols": [0, 4096, 8192]}
    assert gbblas.crt_blocks(8192, 8192, 2, 152) == {"rows": [0, 8192], "cols": [0, 4096, 8192]}
    assert gbblas.crt_blocks(4096, 4096, 3, 152) == {"rows": [0, 4096], "cols": [0, 2048, 4096]}
    assert gbblas.crt_blocks(12288, 12288, 3, 152) == {"rows": [0, 12288], "cols": [0, 768, 10752, 12288]}
    assert gbblas.crt_blocks(300, 1100, 1, 152) == {"rows": [0, 300], "cols": [0, 1100]}
    with pytest.raises(gbblas.GBError):
        gbblas.crt_blocks(0, 8, 2, 152)


@pytest.mark.parametrize("sms", [2, 16, 132, 152])
def test_crt_blocks_match_restatement(sms):
    g = __import__("numpy").random.default_rng(sms)
    for _ in range(300):
        M, N = (int(x) for x in g.integers(1, 40000, 2))
        panels, host = int(g.integers(0, 6)), bool(g.integers(0, 2))
        got = gbblas.crt_blocks(M, N, panels, sms, host)
        assert got == _crt_blocks_restated(M, N, panels, sms, host), (M, N, panels, sms, host)
        assert got["rows"][-1] == M and got["cols"][-1] == N
        assert all(b % 256 == 0 for b in got["rows"][:-1] + got["cols"][:-1])


def test_only_the_c_abi_is_exported():
    """The dynamic symbol table is exactly the header's gb_* functions (internal C++ hidden)."""
    import subprocess
    out = subprocess.run(["nm", "-D", "--defined-only", gbblas.LIB_PATH], capture_output=True, text=True)
    if out.returncode != 0:
        pytest.skip("nm unavailable")
    syms = {line.split()[-1] for line in out.stdout.splitlines() if line.strip()}
    assert syms == set(declared_functions()), sorted(syms ^ set(declared_functions()))[:10]


def test_jmul_prefetch_hints_are_validated():
    """jmul!'s Val prefetch distances and localities are accepted and checked before any GPU work."""
    import torch
    D = torch.zeros(2, 2, dtype=torch.float64)
    with pytest.raises(ValueError):
        gbblas.jmul_(D, D, D, a_prefetch=-1)
    with pytest.raises(ValueError):
        gbblas.jmul_(D, D, D, a_loc=4)
    with pytest.raises(ValueError):
        gbblas.jmul_(D, D, D, 7, 7, 3, 3, 9)


def test_tc_tuning_table_roundtrip_and_validation():
    """The tensor-core tuning table (no GPU work): defaults, set/get per kind and size class,
    invalid combinations refused, NULL restoring the default."""
    import ctypes
    from gbblas import _lib, tuning
    L = _lib.lib()
    assert [tuning.size_class(m, n) for m, n in ((1, 1), (2048, 100), (2049, 5), (8192, 8192), (8193, 1))] == \
        [0, 0, 1, 1, 2]
    for kind in _lib.TC_KINDS:
        for cls in range(_lib.TC_SIZE_CLASSES):
            d = tuning.default_tuning(kind, cls)
            # CRT products above 2048 columns default to three column panels
            panels = 3 if (kind == "ozaki_crt" and cls > 0) else 0
            assert (d.engine, d.band, d.tma_store, d.panels) == (2, 8, 0, panels)
            assert tuning.get_tuning(kind, cls).as_dict() == d.as_dict()
    tuning.set_tuning("f32", 1, {"engine": 2, "band": 16, "tma_store": 1})
    assert tuning.get_tuning("f32", 1).as_dict() == {"engine": 2, "band": 16, "tma_store": 1, "panels": 0}
    assert tuning.get_tuning("f32", 0).as_dict()["band"] == 8
    tuning.set_tuning("ozaki_crt", 2, {"engine": 2, "band": 4, "panels": 4})
    assert tuning.get_tuning("ozaki_crt", 2).as_dict() == {"engine": 2, "band": 4, "tma_store": 0, "panels": 4}
    bad = [("ozaki_crt", {"engine": 1, "band": 8}), ("f32", {"engine": 3, "band": 8}),
           ("f32", {"engine": 2, "band": 0}), ("f32", {"engine": 2, "band": 65}),
           ("ozaki_slices", {"engine": 2, "band": 8, "tma_store": 1}),
           ("adjoint", {"engine": 1, "band": 8, "tma_store": 1}),
           ("ozaki_crt", {"engine": 2, "band": 8, "panels": 5}), ("ozaki_crt", {"engine": 2, "band": 8, "panels": -1}),
           ("f32", {"engine": 2, "band": 8, "panels": 2}), ("ozaki_slices", {"engine": 2, "band": 8, "panels": 2})]
    for kind, d in bad:
        t = _lib.TcTuning.from_dict(d)
        assert L.gb_set_tc_tuning(_lib.TC_KINDS[kind], 0, ctypes.byref(t)) == _lib.GB_ERR_INVALID_VALUE, (kind, d)
    assert L.gb_set_tc_tuning(9, 0, None) == _lib.GB_ERR_INVALID_VALUE
    assert L.gb_set_tc_tuning(2, 3, None) == _lib.GB_ERR_INVALID_VALUE
    t = _lib.TcTuning()
    assert L.gb_tc_default_tuning(1, 3, ctypes.byref(t)) == _lib.GB_ERR_INVALID_VALUE
    tuning.set_tuning("f32", 1, None)
    tuning.set_tuning("ozaki_crt", 2, None)
    assert tuning.get_tuning("f32", 1).as_dict() == tuning.default_tuning("f32", 1).as_dict()
    assert tuning.get_tuning("ozaki_crt", 2).as_dict() == tuning.default_tuning("ozaki_crt", 2).as_dict()
