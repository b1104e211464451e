"""The cuRAND MTGP32 mode of the domino, lozenge, rectangle-triangle and bibone sweeps
(RT_RNG_MTGP): the random stream of the reference's CUDA build (DominoTiler.cpp:51-66,
dominokernel*.cu; LozengeTiler.cpp:71-80, lozengekernel.cu; RectTriangleTiler.cpp:75-85,
recttrianglekernel.cu; TriangleDimerTiler.cpp:279-291, triangledimerkernel.cu).

cuRAND's generator is library code: the oracle does not restate it but takes its draws as
data (rt_domino_mtgp_draws: the curand_uniform value each candidate site receives in the
reference's 8 x 8 block geometry) and replays the reference's CUDA rotate kernels and host
loops on them.  On CPU, the mode's acceptance intervals over the float draw's bit pattern are
checked against the CUDA kernels' own float/double expressions."""
import ctypes as C

import numpy as np
import pytest

RULES = [(0, 0.7, 1.0), (1, 1.0, 1.0), (2, 0.7, 1.0), (2, 1.0, 0.5), (3, 1.0, 0.5), (3, 0.37, 2.3)]
NAMES = {0: "plain", 1: "cftp", 2: "twoperiodic", 3: "cftp_twoperiodic"}
ONE = 0x3F800000  # bit pattern of 1.0f; curand_uniform returns values in (0, 1]


@pytest.mark.parametrize("rule,a,b", RULES)
def test_mtgp_rule_intervals_decide_as_the_cuda_kernels(rt, orc, rule, a, b):
    table = np.zeros(16, np.uint32)
    assert rt.lib().rt_domino_rule_table(rule, rt.RNG_MODES["mtgp"], a, b, table.ctypes.data) == rt.RT_OK
    rng = np.random.default_rng(1000 + rule)
    for c in range(4):
        i, t = 2 + (c & 1), c >> 1
        lo_up, w_up, lo_dn, w_dn = (int(x) for x in table[4 * c: 4 * c + 4])
        for e, lo, w, new in ((3, lo_up, w_up, 12), (12, lo_dn, w_dn, 3)):
            edges = {lo - 1, lo, lo + w - 1, lo + w, 1, ONE, 0x3F000000, 0x3F4CCCCC, 0x3F4CCCCD}
            bits = np.array(sorted(u for u in edges if 1 <= u <= ONE), np.uint32)
            bits = np.concatenate([bits, rng.integers(1, ONE + 1, 200_000, dtype=np.uint32),
                                   rng.integers(0x3E000000, ONE + 1, 200_000, dtype=np.uint32)])
            want = orc.rotate_cuda(bits.view(np.float32), e, rule, i, t, a, b) == new
            mine = ((bits.astype(np.uint64) - lo) % 2**32) < w
            assert np.array_equal(mine, want), (rule, c, e, bits[mine != want][:4])


def test_mtgp_two_periodic_rule_is_the_cuda_kernels_not_the_opencl_ones(rt, orc):
    """dominokerneltwoperiodic.cu divides the draw by the double 0.8 and rounds to float; the
    .cl kernel divides by the float 0.8 in float.  The two thresholds differ by an ulp for some
    draws, which decides a flip when the weight ratio equals the larger one: with b = 1 the up
    move at an odd row of colour 1 has ratio float(a^2), so a = sqrt(threshold) builds such a
    case.  There the MTGP table decides as the CUDA kernel and the TinyMT table as the .cl one."""
    u = np.arange(1 << 20, int(0.8 * 2**23), dtype=np.int64)
    rd = (u.astype(np.float64) / 2**23).astype(np.float32)  # exact: u23 * 2^-23
    cu = (rd.astype(np.float64) / 0.8).astype(np.float32)
    cl = rd / np.float32(0.8)
    for k in np.nonzero(cu != cl)[0]:
        r = max(cu[k], cl[k])
        a = float(np.sqrt(np.float64(r)))
        if np.float32(a * a) == r:
            break
    else:
        pytest.fail("no separating draw")
    c = 3  # odd row, colour 1
    tiny = np.zeros(16, np.uint32)
    mtgp = np.zeros(16, np.uint32)
    assert rt.lib().rt_domino_rule_table(2, rt.RNG_MODES["tinymt"], a, 1.0, tiny.ctypes.data) == 0
    assert rt.lib().rt_domino_rule_table(2, rt.RNG_MODES["mtgp"], a, 1.0, mtgp.ctypes.data) == 0
    flip_cl = ((int(u[k]) - int(tiny[4 * c])) % 2**32) < int(tiny[4 * c + 1])
    bits = int(rd[k:k + 1].view(np.uint32)[0])
    flip_cu = ((bits - int(mtgp[4 * c])) % 2**32) < int(mtgp[4 * c + 1])
    assert flip_cu == bool(r > cu[k]) and flip_cl == bool(r > cl[k])
    assert flip_cu != flip_cl
    assert (orc.rotate_cuda(rd[k:k + 1], 3, 2, 3, 1, a, 1.0)[0] == 12) == flip_cu


def _aztec(rt, order):
    D = rt.DominoTiler
    d = D.AztecDiamond(order)
    return D.MaxTiling(d), D.MinTiling(d)


def _mixed(rt, orc, order):
    """A tiling away from the extremal ones (which have few flippable sites): the max tiling
    after 400 half-sweeps of the oracle's TinyMT walk."""
    t, _ = _aztec(rt, order)
    orc.walk_tinymt(t, rt.side_of(t), 400, 5, 1, 1.0, 1.0)
    return t


@pytest.mark.gpu
def test_mtgp_draws_are_deterministic_uniforms(rt):
    n, launches = 40, 10
    a = rt.mtgp_draws(n, 34893, launches)
    b = rt.mtgp_draws(n, 34893, launches)
    c = rt.mtgp_draws(n, 34894, launches)
    assert a.shape == (launches, n - 2, n // 2 - 2)
    assert np.array_equal(a, b) and not np.array_equal(a, c)
    assert a.min() > 0.0 and a.max() <= 1.0
    assert abs(float(a.mean()) - 0.5) < 0.02
    assert len(np.unique(a)) > 0.99 * a.size


@pytest.mark.gpu
@pytest.mark.parametrize("rule,a,b", RULES)
def test_mtgp_walk_equals_the_reference_cuda_path_on_its_draws(rt, orc, rule, a, b):
    start = _mixed(rt, orc, 9)
    n = rt.side_of(start)
    steps, seed = 150, 34893  # Examples/MinimalDominoEx.cpp walks with seed 34893
    want = start.copy()
    orc.walk_draws(want, n, rt.mtgp_draws(n, seed, steps), steps, seed, rule, a, b)
    got = start.copy()
    rt.DominoTiler(rule=NAMES[rule], rng="mtgp", a=a, b=b).Walk(got, steps, seed)
    assert np.array_equal(got, want)
    assert (got != start).sum() > 8


@pytest.mark.gpu
def test_mtgp_epochs_and_load_mtgp_equal_the_reference_cuda_path(rt, orc):
    start = _mixed(rt, orc, 8)
    n = rt.side_of(start)
    steps, seeds = [96, 48, 32], [7, 123456789, 2**31 + 5]
    draws = np.concatenate([rt.mtgp_draws(n, s, k) for k, s in zip(steps, seeds)])
    want = start.copy()
    orc.walk_epochs_draws(want, n, draws, steps, seeds, 0)
    tiler = rt.DominoTiler()
    tiler.LoadMTGP()
    got = start.copy()
    tiler.Walk(got, steps, seeds)
    assert np.array_equal(got, want)
    assert (got != start).sum() > 8


@pytest.mark.gpu
@pytest.mark.parametrize("rule,a,b", [(1, 1.0, 1.0), (3, 1.0, 0.5)])
def test_mtgp_cftp_equals_the_reference_driver_on_its_draws(rt, orc, rule, a, b):
    """Examples/AztecDiamondCftpEx.cpp:51-77: epochs prepended with doubled steps and fresh
    seeds from mt19937(345903) until the coupled max/min chains agree."""
    tmax, tmin = _aztec(rt, 6)
    n = rt.side_of(tmax)
    driver_seed, first, max_attempts = 345903, 16, 24
    drv = iter(orc.mt19937(driver_seed, 64))
    steps, seeds = [first], [int(next(drv))]
    for attempt in range(1, max_attempts + 1):
        draws = np.concatenate([rt.mtgp_draws(n, s, k) for k, s in zip(steps, seeds)])
        top, bot = tmax.copy(), tmin.copy()
        orc.walk_epochs_draws(top, n, draws, steps, seeds, rule, a, b)
        orc.walk_epochs_draws(bot, n, draws, steps, seeds, rule, a, b)
        if np.array_equal(top, bot):
            break
        steps.insert(0, steps[-1] * 2)
        seeds.insert(0, int(next(drv)))
    else:
        pytest.fail("oracle driver did not coalesce")
    assert attempt > 1  # the look-back grew at least once
    got, stats = rt.DominoTiler(rule=NAMES[rule], rng="mtgp", a=a, b=b).cftp(tmax, tmin, driver_seed=driver_seed,
                                                                             first_steps=first,
                                                                             max_attempts=max_attempts)
    assert stats["attempts"] == attempt
    assert np.array_equal(got, top)


@pytest.mark.gpu
def test_mtgp_walk_with_host_threaded_seeding(rt, orc):
    """Order 128: 33 x 17 = 561 block generators, seeded from several host threads."""
    tmax, _ = _aztec(rt, 128)
    n = rt.side_of(tmax)
    assert ((n - 2 + 7) // 8) * ((n // 2 - 2 + 7) // 8) >= 512
    steps, seed = 8, 99
    orc.walk_tinymt(tmax, n, 200, 5, 1, 1.0, 1.0)
    want = tmax.copy()
    orc.walk_draws(want, n, rt.mtgp_draws(n, seed, steps), steps, seed, 1, 1.0, 1.0)
    got = tmax.copy()
    rt.DominoTiler(rule="cftp", rng="mtgp").Walk(got, steps, seed)
    assert np.array_equal(got, want)
    assert (got != tmax).sum() > 8


@pytest.mark.gpu
def test_mtgp_sampler_refuses_unseeded_runs_and_the_resident_engine(rt):
    tmax, _ = _aztec(rt, 6)
    n = rt.side_of(tmax)
    s = rt.DominoSampler(n, 1, rt.DominoTiler(rng="mtgp"))
    s.load(0, tmax)
    colours = np.zeros(4, np.uint8)
    assert rt.lib().rt_dm_sampler_run(s.h, colours.ctypes.data, 4) == rt.RT_ERR_INVALID_ARGUMENT
    assert rt.lib().rt_dm_sampler_seed(s.h, 5) == rt.RT_OK
    assert rt.lib().rt_dm_sampler_run(s.h, colours.ctypes.data, 4) == rt.RT_OK
    s.close()
    with pytest.raises(rt.RTError):
        rt.DominoSampler(n, 1, rt.DominoTiler(rng="mtgp", engine=2))
    with pytest.raises(rt.RTError):  # the reference's q kernel has no CUDA build to match
        rt.LozengeTiler(rng="mtgp", q=0.9).Walk(rt.LozengeTiler.MaxTiling(rt.LozengeTiler.Hexagon(3)), 4, 1)


@pytest.mark.gpu
def test_cpp_dropin_load_mtgp_walk_equals_the_reference_cuda_path(rt, orc, tmp_path):
    """tests/cpp/dropin_walk.cpp calls LoadMTGP and Walk(T, 100, 34893) through the C++
    header, as the reference's CUDA examples do."""
    import shutil
    import subprocess
    from pathlib import Path

    if not shutil.which("g++"):
        pytest.skip("no g++")
    root = Path(__file__).resolve().parent.parent
    exe = tmp_path / "dropin_walk"
    libdir = str(rt.LIB_PATH.parent)
    subprocess.run(["g++", "-std=c++17", "-O1", f"-I{root / 'include'}", str(root / "tests/cpp/dropin_walk.cpp"),
                    f"-L{libdir}", "-l:librt_tilings.so", f"-Wl,-rpath,{libdir}", "-o", str(exe)], check=True)
    order = 7
    out = subprocess.run([str(exe), str(order)], check=True, capture_output=True, text=True).stdout
    got = np.array([int(x) for x in out.split()], np.int32)
    tmax, _ = _aztec(rt, order)
    n = rt.side_of(tmax)
    want = tmax.copy()
    orc.walk_draws(want, n, rt.mtgp_draws(n, 34893, 100), 100, 34893, 0)
    assert np.array_equal(got, want)


def _lz_mixed(rt, orc, side):
    L = rt.LozengeTiler
    d = L.Hexagon(side)
    tmax, tmin = L.MaxTiling(d), L.MinTiling(d)
    t = tmax.copy()
    orc.lz_walk_tinymt(t, rt.side_of(t), 300, 5)
    return t, tmax, tmin


@pytest.mark.gpu
def test_mtgp_lozenge_walk_equals_the_reference_cuda_path_on_its_draws(rt, orc):
    start, _, _ = _lz_mixed(rt, orc, 7)
    n = rt.side_of(start)
    steps, seed = 120, 2**33 + 17  # a seed beyond 32 bits: generator k gets seed + k in full
    want = start.copy()
    orc.lz_walk_draws(want, n, rt.lozenge_mtgp_draws(n, seed, steps), steps, seed)
    got = start.copy()
    tiler = rt.LozengeTiler()
    tiler.LoadMTGP()
    tiler.Walk(got, steps, seed)
    assert np.array_equal(got, want)
    assert (got != start).sum() > 8
    draws = rt.lozenge_mtgp_draws(n, seed, 2)
    assert draws.shape == (2, n, n // 3) and draws.min() > 0 and draws.max() <= 1


@pytest.mark.gpu
def test_mtgp_lozenge_cftp_equals_epochs_of_reference_walks(rt, orc):
    """rt_lozenge_cftp: every epoch is one reference Walk(t, steps_k, seed_k) of both chains,
    seeds from mt19937(driver_seed), look-back prepending 2 * steps.back()."""
    _, tmax, tmin = _lz_mixed(rt, orc, 3)
    n = rt.side_of(tmax)
    driver_seed, first, max_attempts = 4242, 4, 30
    drv = iter(orc.mt19937(driver_seed, 64))
    steps, seeds = [first], [int(next(drv))]
    for attempt in range(1, max_attempts + 1):
        top, bot = tmax.copy(), tmin.copy()
        for k, sd in zip(steps, seeds):
            d = rt.lozenge_mtgp_draws(n, sd, k)
            orc.lz_walk_draws(top, n, d, k, sd)
            orc.lz_walk_draws(bot, n, d, k, sd)
        if np.array_equal(top, bot):
            break
        steps.insert(0, steps[-1] * 2)
        seeds.insert(0, int(next(drv)))
    else:
        pytest.fail("oracle driver did not coalesce")
    assert attempt > 1
    got, stats = rt.LozengeTiler(rng="mtgp").cftp(tmax, tmin, driver_seed=driver_seed, first_steps=first,
                                                  max_attempts=max_attempts)
    assert stats["attempts"] == attempt
    assert np.array_equal(got, top)


@pytest.mark.gpu
@pytest.mark.parametrize("weights", [None, [1.3, 0.7, 1.1, 0.9, 1.6, 0.8, 1.2, 0.5, 1.4]])
def test_mtgp_recttri_walk_equals_the_reference_cuda_path_on_its_draws(rt, orc, weights):
    R = rt.RectTriangleTiler
    start = R.maxHex(6)
    n = rt.side_of(start)
    orc.rt_walk_tinymt(start, n, 200, 3, weights)  # away from the extremal hexagon
    steps, seed = 90, 8675309
    want = start.copy()
    orc.rt_walk_draws(want, n, rt.recttri_mtgp_draws(n, seed, steps), steps, seed, weights)
    tiler = R(weights=weights)
    tiler.LoadMTGP()
    got = start.copy()
    tiler.Walk(got, steps, seed)
    assert np.array_equal(got, want)
    assert (got != start).sum() > 8


@pytest.mark.gpu
def test_mtgp_bibone_walk_equals_the_reference_cuda_path_on_its_draws(rt, orc):
    T = rt.TriangleDimerTiler
    start = T.RhombusBrick(14, 14)
    n = rt.side_of(start)
    orc.td_walk_tinymt(start, n, 300, 3)  # away from the brick pattern
    steps, seed = 120, 31337
    want = start.copy()
    orc.td_walk_draws(want, n, rt.td_mtgp_draws(n, seed, steps), steps, seed)
    tiler = T()
    tiler.LoadMTGP()
    got = start.copy()
    tiler.Walk(got, steps, seed)
    assert np.array_equal(got, want)
    assert (got != start).sum() > 8


def test_mtgp_entry_points_check_their_arguments_before_any_cuda_call(rt):
    """Bad sizes are refused on the host (no device needed), and the q-weighted lozenge rule has
    no MTGP mode: the reference's q kernel has no CUDA build to match."""
    out = np.zeros(64, np.float32)
    lib = rt.lib()
    assert lib.rt_domino_mtgp_draws(7, 1, 1, out.ctypes.data) == rt.RT_ERR_INVALID_ARGUMENT  # odd side
    assert lib.rt_domino_mtgp_draws(8, 1, -1, out.ctypes.data) == rt.RT_ERR_INVALID_ARGUMENT
    assert lib.rt_domino_mtgp_draws(8, 1, 1, None) == rt.RT_ERR_INVALID_ARGUMENT
    assert lib.rt_lozenge_mtgp_draws(10, 1, 1, out.ctypes.data) == rt.RT_ERR_INVALID_ARGUMENT  # not 3k
    assert lib.rt_recttri_mtgp_draws(8, 1, 1, out.ctypes.data) == rt.RT_ERR_INVALID_ARGUMENT
    assert lib.rt_td_mtgp_draws(9, 1, 1, out.ctypes.data) == rt.RT_ERR_INVALID_ARGUMENT
    L = rt.LozengeTiler
    t = L.MaxTiling(L.Hexagon(3))
    o = rt.LozengeTiler(rng="mtgp", q=0.9).opts()
    status = lib.rt_lozenge_walk(t.ctypes.data, rt.side_of(t), 4, 1, C.byref(o))
    assert status == rt.RT_ERR_INVALID_ARGUMENT
    assert "uniform rule" in lib.rt_last_error().decode()


def _write_tinymtdc(path, params) -> None:
    """A parameter file in the TinyMTDC text format LoadTinyMT reads (file_reader.cpp:22-38):
    a '#' header line, then one line per set with mat1, mat2, tmat in hex after the 3rd, 4th
    and 5th comma."""
    lines = ["# synthetic TinyMTDC parameter sets"]
    for k, (m1, m2, tm) in enumerate(params):
        lines.append(f"{k:08x},32,0,{m1:08x},{m2:08x},{tm:08x},0")
    path.write_text("\n".join(lines) + "\n")


@pytest.mark.gpu
@pytest.mark.parametrize("model,gold,case_name", [
    ("lozenge", "lozenge_ref_cases.json", "lz_walk_hex5_0_paramtable"),
    ("recttri", "recttri_ref_cases.json", "rt_walk_hex5_min_paramtable"),
    ("bibone", "bibone_ref_cases.json", "td_walk_cone7_0_paramtable"),
])
def test_cpp_dropin_load_tinymt_file_walk_equals_the_reference(rt, tmp_path, model, gold, case_name):
    """tests/cpp/dropin_tinymt_file.cpp reads a TinyMTDC parameter file with LoadTinyMT and
    walks, for the three tilers whose LoadTinyMT the reference's OpenCL path has
    (LozengeTiler.cpp:161-164, RectTriangleTiler.cpp:22-25, TriangleDimerTiler.cpp:24-27);
    the result equals the reference's own kernels run with the same table."""
    import json
    import shutil
    import subprocess
    from pathlib import Path

    if not shutil.which("g++"):
        pytest.skip("no g++")
    root = Path(__file__).resolve().parent.parent
    case = next(c for c in json.loads((root / "tests/golden" / gold).read_text())["cases"] if c["name"] == case_name)
    exe = tmp_path / "dropin_tinymt_file"
    libdir = str(rt.LIB_PATH.parent)
    subprocess.run(["g++", "-std=c++17", "-O1", f"-I{root / 'include'}", str(root / "tests/cpp/dropin_tinymt_file.cpp"),
                    f"-L{libdir}", "-l:librt_tilings.so", f"-Wl,-rpath,{libdir}", "-o", str(exe)], check=True)
    pfile = tmp_path / "params.txt"
    _write_tinymtdc(pfile, case["params"])
    out = subprocess.run([str(exe), model, str(pfile), str(len(case["params"])), str(case["steps"]), str(case["seed"])],
                         check=True, capture_output=True, text=True).stdout
    got = np.array([int(x) for x in out.split()], np.int32)
    assert np.array_equal(got, case["expected"])


def test_tinymt_file_reader_reads_the_written_sets(rt, tmp_path):
    """The Python reader of the TinyMTDC format returns the sets written (the C++ header's
    reader follows the same rules)."""
    params = [[0x8f7011ee, 0xfc78ff1f, 0x3793fdff], [1, 2, 3], [0xffffffff, 0, 0x10]]
    pfile = tmp_path / "params.txt"
    _write_tinymtdc(pfile, params)
    assert rt.read_tinymt_params(pfile, 3).tolist() == params
