"""The autotuner: its table format and lookup (CPU), and on the GPU that every launch shape
it chooses between gives the same chains (the draws are keyed by site, not by thread), and
that a tuning pass writes a table the samplers then follow."""
import numpy as np
import pytest


def test_tune_table_lookup(rt, tmp_path):
    p = tmp_path / "tune.txt"
    p.write_text("# comment\n"
                 "domino 6 300 2 tinymt 2 152 768 1.5  # order 128\n"
                 "domino 301 32768 2 tinymt 3 0 0\n"
                 "domino 6 32768 1 fast 1 0 0\n")
    rt.tune_load(p)
    try:
        assert rt.tune_lookup(262, 2, "tinymt") == {"engine": 2, "bands": 152, "threads": 768}
        assert rt.tune_lookup(2054, 2, "tinymt") == {"engine": 3, "bands": 0, "threads": 0}
        assert rt.tune_lookup(2054, 1, "fast") == {"engine": 1, "bands": 0, "threads": 0}
        assert rt.tune_lookup(2054, 4, "tinymt") is None
    finally:
        rt.tune_clear()
    assert rt.tune_lookup(262, 2, "tinymt") is None


@pytest.mark.parametrize("line", ["domino 6 300 2 tinymt 2 152\n", "lozenge 6 300 2 tinymt 2 0 0\n",
                                  "domino 6 300 2 philox 2 0 0\n", "domino 6 300 2 tinymt 2 0 100\n"])
def test_tune_table_rejects_malformed_lines(rt, tmp_path, line):
    p = tmp_path / "bad.txt"
    p.write_text(line)
    with pytest.raises(rt.RTError) as e:
        rt.tune_load(p)
    assert e.value.status == rt.RT_ERR_INVALID_ARGUMENT


def _walk(rt, rng, shape, tmax, tmin, steps=300, seed=77):
    n = rt.side_of(tmax)
    s = rt.DominoSampler(n, 2, rt.DominoTiler(rule="cftp_twoperiodic", rng=rng, a=1.0, b=0.5))
    s.load(0, tmax)
    s.load(1, tmin)
    s.set_launch(*shape)
    info = s.engine_info()
    if rng == "tinymt":
        s.seed(seed)
        s.run(rt.mt19937_colours(seed, steps))
    else:
        s.run_fast(seed, 0, steps)
    out = (s.store(0), s.store(1))
    s.close()
    return out, info


@pytest.mark.gpu
@pytest.mark.parametrize("rng", ["tinymt", "fast"])
def test_every_launch_shape_gives_the_same_chains(rt, rng):
    D = rt.DominoTiler
    d = D.AztecDiamond(200)
    tmax, tmin = D.MaxTiling(d), D.MinTiling(d)
    ref, info = _walk(rt, rng, (1, 0, 0), tmax, tmin)
    assert info["engine"] == 1
    seen = set()
    for shape in [(3, 0, 0), (2, 0, 0), (2, 152, 512), (2, 114, 768), (2, 76, 1024), (2, 40, 896)]:
        got, info = _walk(rt, rng, shape, tmax, tmin)
        seen.add((info["engine"], info["bands"], info["threads"]))
        assert np.array_equal(got[0], ref[0]) and np.array_equal(got[1], ref[1]), shape
    assert len(seen) >= 5  # the shapes really differ


@pytest.mark.gpu
def test_tuning_pass_writes_a_table_the_sampler_follows(rt, tmp_path):
    from randomtilingspublic_gb300 import autotune

    rt.tune_clear()
    entries = autotune.tune_domino(rt, [24, 48], chains_list=(2,), rngs=("fast",), half_sweeps=64, log=lambda m: None)
    assert len(entries) == 2 and entries[0]["n_hi"] + 1 == entries[1]["n_lo"]
    path = tmp_path / "tune.txt"
    autotune.write_table(entries, path)
    rt.tune_load(path)
    try:
        D = rt.DominoTiler
        d = D.AztecDiamond(48)
        tmax, tmin = D.MaxTiling(d), D.MinTiling(d)
        got, info = _walk(rt, "fast", (0, 0, 0), tmax, tmin)
        best = entries[1]
        assert info["tuned"] and info["engine"] == best["engine"]
        ref, _ = _walk(rt, "fast", (1, 0, 0), tmax, tmin)
        assert np.array_equal(got[0], ref[0]) and np.array_equal(got[1], ref[1])
    finally:
        rt.tune_clear()
