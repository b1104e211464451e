"""The model-generic C entry points (rt_walk, rt_walk_epochs, rt_cftp) dispatch to the
per-model functions: the same inputs give bit-identical results, and models without the
requested operation are refused (checked without a GPU)."""
import ctypes as C

import numpy as np
import pytest


def _walk(rt, model, state, n, steps, seed, opts, weights=None):
    out = np.ascontiguousarray(state, np.int32).copy()
    w = None if weights is None else np.ascontiguousarray(weights, np.float64)
    st = rt.lib().rt_walk(model, rt._ptr(out), n, steps, seed, None if w is None else w.ctypes.data, C.byref(opts))
    return st, out


def test_refusals_need_no_gpu(rt):
    lib = rt.lib()
    t = np.zeros(36, np.int32)
    o = rt.DominoTiler(rule="cftp", rng="fast").opts()
    assert lib.rt_walk(9, rt._ptr(t), 6, 1, 1, None, C.byref(o)) == rt.RT_ERR_INVALID_ARGUMENT
    steps, seeds = np.array([1], np.int64), np.array([1], np.int64)
    assert lib.rt_walk_epochs(rt.RT_MODEL_LOZENGE, rt._ptr(t), 6, rt._ptr(steps), rt._ptr(seeds), 1,
                              C.byref(o)) == rt.RT_ERR_INVALID_ARGUMENT
    stats = rt.CftpStats()
    for model in (rt.RT_MODEL_RECTTRI, rt.RT_MODEL_BIBONE, 9):
        assert lib.rt_cftp(model, rt._ptr(t), rt._ptr(t), 6, 1, 8, 0, 2, None, C.byref(o), rt._ptr(t),
                           C.byref(stats)) == rt.RT_ERR_INVALID_ARGUMENT
    assert "monotone" in lib.rt_last_error().decode() or "model" in lib.rt_last_error().decode()


@pytest.mark.gpu
def test_rt_walk_equals_the_per_model_walks(rt):
    D, L, R, T, S = rt.DominoTiler, rt.LozengeTiler, rt.RectTriangleTiler, rt.TriangleDimerTiler, rt.SixVertexTiler
    # domino, TinyMT mode (the reference's)
    dt = D(rule="cftp")
    t = D.MaxTiling(D.AztecDiamond(12))
    a = t.copy()
    dt.Walk(a, 60, 7)
    st, b = _walk(rt, rt.RT_MODEL_DOMINO, t, rt.side_of(t), 60, 7, dt.opts())
    assert st == rt.RT_OK and np.array_equal(a, b)
    # lozenge, fast mode
    lt = L(rng="fast", fast_stream=1)
    t = L.MaxTiling(L.Hexagon(6))
    a = t.copy()
    lt.Walk(a, 90, 3)
    st, b = _walk(rt, rt.RT_MODEL_LOZENGE, t, rt.side_of(t), 90, 3, lt.opts())
    assert st == rt.RT_OK and np.array_equal(a, b)
    # rectangle-triangle with weights
    w = [1.0, 0.8, 1.2, 0.9, 1.1, 1.0, 0.7, 1.3, 1.0]
    rtt = R(rng="fast", fast_stream=2, weights=w)
    t = R.minHex(5)
    a = t.copy()
    rtt.Walk(a, 120, 5)
    st, b = _walk(rt, rt.RT_MODEL_RECTTRI, t, rt.side_of(t), 120, 5, rtt.opts(), w)
    assert st == rt.RT_OK and np.array_equal(a, b) and not np.array_equal(a, t)
    # bibone
    tdt = T(rng="fast", fast_stream=4)
    t = T.RhombusBrick(12, 12)
    a = t.copy()
    tdt.Walk(a, 90, 9)
    st, b = _walk(rt, rt.RT_MODEL_BIBONE, t, rt.side_of(t), 90, 9, tdt.opts())
    assert st == rt.RT_OK and np.array_equal(a, b)
    # six-vertex: height function, n = side - 1, steps are sweeps
    svt = S(1.0, 1.0, 1.5, fast_stream=5)
    h = S.MaxHeight(10)
    a = h.copy()
    svt.Walk(a, 40, 11)
    st, b = _walk(rt, rt.RT_MODEL_SIX_VERTEX, h, rt.side_of(h) - 1, 40, 11, svt.opts(), [1.0, 1.0, 1.5])
    assert st == rt.RT_OK and np.array_equal(a, b) and not np.array_equal(a, h)


@pytest.mark.gpu
def test_rt_cftp_equals_the_per_model_cftp(rt):
    D, L, S = rt.DominoTiler, rt.LozengeTiler, rt.SixVertexTiler
    lib = rt.lib()
    stats = rt.CftpStats()
    cases = []
    d = D.AztecDiamond(6)
    cases.append((rt.RT_MODEL_DOMINO, D(rule="cftp", rng="fast", fast_stream=3), D.MaxTiling(d), D.MinTiling(d), None))
    h = L.Hexagon(4)
    cases.append((rt.RT_MODEL_LOZENGE, L(rng="fast", fast_stream=4), L.MaxTiling(h), L.MinTiling(h), None))
    for model, tiler, tmax, tmin, w in cases:
        want, wst = tiler.cftp(tmax, tmin, 21, first_steps=16, schedule=1, max_attempts=16)
        out = np.zeros_like(tmax)
        st = lib.rt_cftp(model, rt._ptr(tmax), rt._ptr(tmin), rt.side_of(tmax), 21, 16, 1, 16, None, C.byref(tiler.opts()),
                         rt._ptr(out), C.byref(stats))
        assert st == rt.RT_OK and np.array_equal(out, want) and stats.attempts == wst["attempts"], model
    svt = S(1.0, 1.0, 1.5, fast_stream=6)
    hmax, hmin = S.MaxHeight(6), S.MinHeight(6)
    want, wst = svt.cftp(hmax, hmin, 17, first_sweeps=8, max_attempts=16)
    abc = np.array([1.0, 1.0, 1.5])
    out = np.zeros_like(hmax)
    st = lib.rt_cftp(rt.RT_MODEL_SIX_VERTEX, rt._ptr(hmax), rt._ptr(hmin), rt.side_of(hmax) - 1, 17, 8, 0, 16,
                     abc.ctypes.data, C.byref(svt.opts()), rt._ptr(out), C.byref(stats))
    assert st == rt.RT_OK and np.array_equal(out, want) and stats.attempts == wst["attempts"]
