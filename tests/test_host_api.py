"""CPU tests of librt_tilings.so: the host utilities against the oracle and the reference
vectors, the rule tables against the reference decision over every draw, the exported
symbols against include/rt_tilings.h, and argument checking (no GPU needed)."""
import ctypes as C
import re
from pathlib import Path

import numpy as np
import pytest

ROOT = Path(__file__).resolve().parent.parent


def test_every_declared_symbol_is_exported(rt):
    header = (ROOT / "include/rt_tilings.h").read_text()
    names = re.findall(r"RT_API\s+[\w\s\*]+?\b(rt_\w+)\s*\(", header)
    assert len(names) >= 30
    lib = rt.lib()
    for name in names:
        assert hasattr(lib, name), name


def test_host_utilities_match_reference_vectors(rt, golden):
    D = rt.DominoTiler
    for hc in golden["host_cases"]:
        d = D.AztecDiamond(hc["order"])
        assert np.array_equal(d, hc["domain"])
        assert np.array_equal(D.MaxTiling(d), hc["max"])
        assert np.array_equal(D.MinTiling(d), hc["min"])
        assert np.array_equal(D.TilingToHeightfunc(hc["max"], d), hc["hf_max"])
    assert np.array_equal(D.MinTiling(D.AztecDiamond(16)), golden["pins"]["min_tiling_aztec16"])
    assert np.array_equal(D.Rectangle(6, 9), golden["pins"]["rectangle_6x9"])


@pytest.mark.parametrize("order", [1, 4, 17, 60])
def test_host_utilities_match_oracle(rt, orc, order):
    D = rt.DominoTiler
    d = D.AztecDiamond(order)
    assert np.array_equal(d, orc.aztec_rectangle(order))
    assert np.array_equal(D.DomainToVertices(d), orc.domain_to_vertices(d))
    for mine, theirs in ((D.MaxTiling, orc.max_tiling), (D.MinTiling, orc.min_tiling)):
        t = mine(d)
        rc, t_o = theirs(d)
        assert rc == 0 and np.array_equal(t, t_o)
        hf = D.TilingToHeightfunc(t, d)
        assert np.array_equal(hf, orc.tiling_to_heightfunc(t, d))
        assert np.array_equal(D.HeightfuncToTiling(hf, d), orc.heightfunc_to_tiling(hf, d))
        assert np.array_equal(D.HeightfuncToTiling(hf, d), t)
        assert np.array_equal(D.TilingToDomain(t), orc.tiling_to_domain(t))


def test_aztec_rectangle_and_rectangle_match_oracle(rt, orc):
    D = rt.DominoTiler
    for n, rm in [(4, [1]), (6, [0, 2]), (9, [1, 3, 5])]:
        assert np.array_equal(D.AztecRectangle(n, rm), orc.aztec_rectangle(n, rm))
    for r, c in [(2, 2), (4, 7), (10, 3)]:
        d = D.Rectangle(r, c)
        assert np.array_equal(d, orc.rectangle(r, c))
        t = D.MaxTiling(d)
        rc, t_o = orc.max_tiling(d)
        assert rc == 0 and np.array_equal(t, t_o)


def test_height_function_is_between_min_and_max(rt):
    D = rt.DominoTiler
    d = D.AztecDiamond(12)
    hmax = D.TilingToHeightfunc(D.MaxTiling(d), d)
    hmin = D.TilingToHeightfunc(D.MinTiling(d), d)
    inside = hmax != np.iinfo(np.int32).max
    assert (hmin[inside] <= hmax[inside]).all() and (hmin[inside] < hmax[inside]).any()


def test_untileable_domain_is_an_error(rt):
    D = rt.DominoTiler
    d = D.Rectangle(3, 3)  # odd area
    with pytest.raises(rt.RTError) as e:
        D.MaxTiling(d)
    assert e.value.status == rt.RT_ERR_NOT_TILEABLE


@pytest.mark.parametrize("rule", [0, 1, 2, 3])
@pytest.mark.parametrize("weights", [(0.7, 1.0), (1.0, 0.5), (0.3, 0.9)])
def test_tinymt_rule_tables_equal_reference_decisions(rt, orc, rule, weights):
    """Every one of the 2^23 draws decides as the reference's float expression does."""
    a, b = weights
    table = np.zeros(16, np.uint32)
    assert rt.lib().rt_domino_rule_table(rule, 0, a, b, table.ctypes.data) == 0
    scan = np.zeros(4, np.uint32)
    for c in range(4):
        assert orc.lib().orc_dm_scan_intervals(rule, c & 1, c >> 1, C.c_double(a), C.c_double(b), scan.ctypes.data) == 0
        lo_up, w_up, lo_dn, w_dn = table[4 * c: 4 * c + 4]
        assert (lo_up, w_up) == (scan[0], scan[1]) or (w_up == 0 and scan[1] == 0)
        assert (lo_dn, w_dn) == (scan[2], scan[3]) or (w_dn == 0 and scan[3] == 0)


@pytest.mark.parametrize("rule", [0, 1, 2, 3])
def test_fast_rule_tables_equal_oracle_at_interval_edges(rt, orc, rule):
    a, b = 1.0, 0.5
    f = orc.lib().orc_dm_rotate_fast
    f.argtypes = [C.c_int, C.c_uint32, C.c_int, C.c_int, C.c_int, C.c_double, C.c_double]
    table = np.zeros(16, np.uint32)
    assert rt.lib().rt_domino_rule_table(rule, 1, a, b, table.ctypes.data) == 0
    for c in range(4):
        lo_up, w_up, lo_dn, w_dn = (int(x) for x in table[4 * c: 4 * c + 4])
        i, t = 2 + (c & 1), c >> 1
        for e, lo, w, new in ((3, lo_up, w_up, 12), (12, lo_dn, w_dn, 3)):
            for u in {lo, lo + w - 1, lo + w, (lo - 1) % 2**32, 0, 2**31 - 1, 2**31, 2**32 - 1}:
                u %= 2**32
                mine = new if ((u - lo) % 2**32) < w else e
                assert f(e, u, rule, i, t, a, b) == mine, (rule, c, e, u)


def test_invalid_arguments_rejected_before_any_gpu_work(rt):
    D = rt.DominoTiler
    t = np.zeros(7 * 7, np.int32)  # odd side
    with pytest.raises(rt.RTError) as e:
        D().Walk(t, 10, 1)
    assert e.value.status == rt.RT_ERR_INVALID_ARGUMENT
    t = np.zeros(8 * 8, np.int32)
    t[10] = 99  # not an edge mask
    with pytest.raises(rt.RTError):
        D().Walk(t, 1, 1)
    with pytest.raises(rt.RTError) as e:
        D(rule="twoperiodic", a=0.0).Walk(np.zeros(64, np.int32), 1, 1)
    assert e.value.status == rt.RT_ERR_INVALID_ARGUMENT
    with pytest.raises(rt.RTError) as e:
        D(rule="plain").cftp(np.zeros(64, np.int32), np.zeros(64, np.int32), 1)
    assert e.value.status == rt.RT_ERR_INVALID_ARGUMENT


def test_tinymt_parameter_file_reader(rt, tmp_path):
    p = tmp_path / "params.txt"
    p.write_text("# header\n# more\ntinymt32dc,0,127,8f7011ee,fc78ff1f,3793fdff,63,0\n"
                 "tinymt32dc,1,127,1,2,3,63,0\n")
    got = rt.read_tinymt_params(p, 2)
    assert got.tolist() == [[0x8F7011EE, 0xFC78FF1F, 0x3793FDFF], [1, 2, 3]]
    with pytest.raises(ValueError):
        rt.read_tinymt_params(p, 3)


def test_cpp_dropin_header_compiles_and_runs(rt, tmp_path):
    """include/rt_tilings.hpp used as the reference's own examples use DominoTiler."""
    import shutil
    import subprocess

    if not shutil.which("g++"):
        pytest.skip("no g++")
    exe = tmp_path / "dropin"
    libdir = str(rt.LIB_PATH.parent)
    subprocess.run(["g++", "-std=c++17", "-O1", f"-I{ROOT / 'include'}", str(ROOT / "tests/cpp/dropin_host.cpp"),
                    f"-L{libdir}", "-l:librt_tilings.so", f"-Wl,-rpath,{libdir}", "-o", str(exe)], check=True)
    out = subprocess.run([str(exe)], check=True, capture_output=True, text=True).stdout
    D = rt.DominoTiler
    d = D.AztecDiamond(5)
    tmax, tmin = D.MaxTiling(d), D.MinTiling(d)
    n = int(np.sqrt(tmax.size))
    assert f"side {n} max {int(tmax.sum())} min {int(tmin.sum())} roundtrip 1" in out
    assert f"untileable status {rt.RT_ERR_NOT_TILEABLE}" in out
    lmax = rt.LozengeTiler.MaxTiling(rt.LozengeTiler.AlmostHexDomain(4, 0))
    rmax = rt.RectTriangleTiler.maxHex(5)
    cone = rt.TriangleDimerTiler.IceCreamCone(6, 0)
    cells = int(rt.TriangleDimerTiler.TilingToDomain(cone).sum())
    assert (f"lozenge {int(np.sqrt(lmax.size))} recttri {int(np.sqrt(rmax.size))} cone {int(np.sqrt(cone.size))} "
            f"cells {cells} asm 5") in out


def test_matrix_text_format_matches_the_reference_bytes(rt, tmp_path):
    """rt_save_matrix writes what the reference's SaveMatrix wrote for maxHex(5) (the committed
    Examples/ExampleOuts/RectTriangle/MaxTiling.txt, kept in tests/golden), and
    rt_load_matrix reads it back."""
    import json

    pin = json.loads((ROOT / "tests/golden/recttri_ref_cases.json").read_text())["format_pin"]
    t = rt.RectTriangleTiler.maxHex(pin["n"])
    path = tmp_path / "max.txt"
    rt.SaveMatrix(t, path)
    assert path.read_text() == pin["text"]
    assert np.array_equal(rt.LoadMatrix(path), t)
    # rows x cols overload and the square overload's truncation to floor(sqrt(size))^2
    rt.SaveMatrix(np.arange(6), tmp_path / "r.txt", rows=2, cols=3)
    assert (tmp_path / "r.txt").read_text() == "0 1 2 \n3 4 5 \n"
    rt.SaveMatrix(np.arange(10), tmp_path / "s.txt")
    assert (tmp_path / "s.txt").read_text() == "0 1 2 \n3 4 5 \n6 7 8 \n"
    (tmp_path / "neg.txt").write_text("-3 12\n7")
    assert rt.LoadMatrix(tmp_path / "neg.txt").tolist() == [3, 12, 7]  # no sign, as the reference
