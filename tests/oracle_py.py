"""ctypes bindings of the oracle (oracle/_build/liboracle.so), the CPU checker of the
library.  Test infrastructure: imported only by tests/, __graft_entry__.smoke() and the
CPU-baseline leg of bench.py."""
from __future__ import annotations

import ctypes as C
import subprocess
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parent.parent
ORACLE_DIR = ROOT / "oracle"
ORACLE_LIB = ORACLE_DIR / "_build" / "liboracle.so"
REF_DIR = ORACLE_DIR / "_ref"

_P = C.c_void_p
_L = C.c_long
_SIG = {
    "orc_dm_aztec_rectangle": (C.c_int, [C.c_int, _P, C.c_int, _P, _L]),
    "orc_dm_rectangle": (C.c_int, [C.c_int, C.c_int, _P, _L]),
    "orc_dm_domain_to_vertices": (None, [_P, C.c_int, _P]),
    "orc_dm_max_tiling": (C.c_int, [_P, C.c_int, _P]),
    "orc_dm_min_tiling": (C.c_int, [_P, C.c_int, _P]),
    "orc_dm_heightfunc_to_tiling": (None, [_P, _P, C.c_int, _P]),
    "orc_dm_tiling_to_heightfunc": (None, [_P, _P, C.c_int, _P]),
    "orc_dm_tiling_to_domain": (None, [_P, C.c_int, _P]),
    "orc_dm_walk_tinymt": (C.c_int, [_P, C.c_int, _L, _L, C.c_int, C.c_double, C.c_double, _P, _L, C.c_int]),
    "orc_dm_walk_epochs_tinymt": (C.c_int, [_P, C.c_int, _P, _P, C.c_int, C.c_int, C.c_double, C.c_double, _P, _L,
                                            C.c_int]),
    "orc_dm_cftp_tinymt": (C.c_int, [_P, _P, C.c_int, _L, _L, C.c_int, C.c_int, C.c_int, C.c_double, C.c_double, _P,
                                     _L, C.c_int, _P, _P]),
    "orc_dm_walk_fast": (C.c_int, [_P, C.c_int, _L, _L, C.c_ulong, C.c_uint, C.c_int, C.c_double, C.c_double,
                                   C.c_int]),
    "orc_dm_cftp_fast": (C.c_int, [_P, _P, C.c_int, C.c_ulong, C.c_uint, _L, C.c_int, C.c_int, C.c_double,
                                   C.c_double, C.c_int, _P, _P]),
    "orc_dm_walk_draws": (C.c_int, [_P, C.c_int, _P, _L, _L, C.c_int, C.c_double, C.c_double]),
    "orc_dm_walk_epochs_draws": (C.c_int, [_P, C.c_int, _P, _P, _P, C.c_int, C.c_int, C.c_double, C.c_double]),
    "orc_dm_rotate_cuda_many": (None, [_P, _L, C.c_int, C.c_int, C.c_int, C.c_int, C.c_double, C.c_double, _P]),
    "orc_mt19937": (None, [C.c_uint, _L, _P]),
    "orc_tinymt_u32": (C.c_uint, [C.c_uint, C.c_uint, C.c_uint, C.c_uint, C.c_int]),
    "orc_philox4x32_10": (None, [_P, _P, _P]),
    "orc_tmt_seed_states": (None, [C.c_uint, _L, _P]),
}

_lib = None


def lib() -> C.CDLL:
    global _lib
    if _lib is None:
        subprocess.run(["make", "-s", "-C", str(ORACLE_DIR)], check=True)
        h = C.CDLL(str(ORACLE_LIB))
        for name, (res, args) in _SIG.items():
            f = getattr(h, name)
            f.restype = res
            f.argtypes = args
        _lib = h
    return _lib


def _i32(a) -> np.ndarray:
    return np.ascontiguousarray(np.asarray(a, dtype=np.int32).ravel())


def _p(a: np.ndarray | None):
    return None if a is None else a.ctypes.data


def _params(params):
    if params is None:
        return None, 0
    p = np.ascontiguousarray(np.asarray(params, dtype=np.uint32).reshape(-1, 3))
    return p, p.shape[0]


def aztec_rectangle(n: int, remove=()) -> np.ndarray:
    m = 2 * n - len(remove) + 6
    buf = np.zeros(m * m, np.int32)
    rm = _i32(list(remove)) if len(remove) else None
    side = lib().orc_dm_aztec_rectangle(n, _p(rm), len(remove), _p(buf), buf.size)
    return buf[: side * side].copy()


def rectangle(rows: int, cols: int) -> np.ndarray:
    m = max(rows, cols) + 6
    buf = np.zeros(m * m, np.int32)
    side = lib().orc_dm_rectangle(rows, cols, _p(buf), buf.size)
    return buf[: side * side].copy()


def _side(a) -> int:
    import math
    return math.isqrt(len(a))


def domain_to_vertices(d) -> np.ndarray:
    d = _i32(d)
    m = _side(d)
    out = np.zeros((m + 1) ** 2, np.int32)
    lib().orc_dm_domain_to_vertices(_p(d), m, _p(out))
    return out


def max_tiling(d):
    d = _i32(d)
    m = _side(d)
    out = np.zeros((m + 1) ** 2, np.int32)
    rc = lib().orc_dm_max_tiling(_p(d), m, _p(out))
    return rc, out


def min_tiling(d):
    d = _i32(d)
    m = _side(d)
    out = np.zeros((m + 1) ** 2, np.int32)
    rc = lib().orc_dm_min_tiling(_p(d), m, _p(out))
    return rc, out


def tiling_to_heightfunc(t, d) -> np.ndarray:
    t, d = _i32(t), _i32(d)
    n = _side(t)
    out = np.zeros(n * n, np.int32)
    lib().orc_dm_tiling_to_heightfunc(_p(t), _p(d), n, _p(out))
    return out


def heightfunc_to_tiling(h, d) -> np.ndarray:
    h, d = _i32(h), _i32(d)
    n = _side(h)
    out = np.zeros(n * n, np.int32)
    lib().orc_dm_heightfunc_to_tiling(_p(h), _p(d), n, _p(out))
    return out


def tiling_to_domain(t) -> np.ndarray:
    t = _i32(t)
    n = _side(t)
    out = np.zeros((n - 1) ** 2, np.int32)
    lib().orc_dm_tiling_to_domain(_p(t), n, _p(out))
    return out


def walk_tinymt(t: np.ndarray, n: int, steps: int, seed: int, rule: int = 0, a=0.7, b=1.0, params=None,
                threads: int = 1) -> None:
    p, cnt = _params(params)
    rc = lib().orc_dm_walk_tinymt(_p(t), n, steps, seed, rule, a, b, _p(p), cnt, threads)
    assert rc == 0


def walk_epochs_tinymt(t: np.ndarray, n: int, steps, seeds, rule: int = 0, a=0.7, b=1.0, params=None,
                       threads: int = 1) -> None:
    st = np.ascontiguousarray(np.asarray(steps, np.int64))
    sd = np.ascontiguousarray(np.asarray(seeds, np.int64))
    p, cnt = _params(params)
    rc = lib().orc_dm_walk_epochs_tinymt(_p(t), n, _p(st), _p(sd), len(st), rule, a, b, _p(p), cnt, threads)
    assert rc == 0


def cftp_tinymt(tmax, tmin, n, driver_seed, first_steps, schedule, max_attempts, rule=1, a=0.7, b=1.0, params=None,
                threads: int = 1):
    tmax, tmin = _i32(tmax), _i32(tmin)
    out = np.zeros_like(tmax)
    total = C.c_long()
    p, cnt = _params(params)
    att = lib().orc_dm_cftp_tinymt(_p(tmax), _p(tmin), n, driver_seed, first_steps, schedule, max_attempts, rule, a,
                                   b, _p(p), cnt, threads, _p(out), C.addressof(total))
    return out, att, total.value


def walk_draws(t: np.ndarray, n: int, draws: np.ndarray, steps: int, seed: int, rule: int = 0, a=0.7,
               b=1.0) -> None:
    """The reference's CUDA-path walk with its MTGP32 draws supplied (steps x (n-2) x (n/2-2))."""
    d = np.ascontiguousarray(draws, np.float32)
    assert d.size == steps * (n - 2) * (n // 2 - 2)
    assert lib().orc_dm_walk_draws(_p(t), n, _p(d), steps, seed, rule, a, b) == 0


def walk_epochs_draws(t: np.ndarray, n: int, draws: np.ndarray, steps, seeds, rule: int = 0, a=0.7, b=1.0) -> None:
    """CUDA-path epochs; draws holds the epochs' draws one after another."""
    st = np.ascontiguousarray(np.asarray(steps, np.int64))
    sd = np.ascontiguousarray(np.asarray(seeds, np.int64))
    d = np.ascontiguousarray(draws, np.float32)
    assert d.size == int(st.sum()) * (n - 2) * (n // 2 - 2)
    assert lib().orc_dm_walk_epochs_draws(_p(t), n, _p(d), _p(st), _p(sd), len(st), rule, a, b) == 0


def rotate_cuda(rd: np.ndarray, e: int, rule: int, i: int, t: int, a=0.7, b=1.0) -> np.ndarray:
    """The CUDA kernels' new state for state e and each float draw in rd."""
    r = np.ascontiguousarray(rd, np.float32)
    out = np.zeros(r.size, np.uint8)
    lib().orc_dm_rotate_cuda_many(_p(r), r.size, e, rule, i, t, a, b, _p(out))
    return out


def mt19937(seed: int, n: int) -> np.ndarray:
    out = np.zeros(n, np.uint32)
    lib().orc_mt19937(seed & 0xFFFFFFFF, n, _p(out))
    return out


def walk_fast(t: np.ndarray, n: int, h0: int, steps: int, seed: int, stream: int = 0, rule: int = 0, a=0.7, b=1.0,
              threads: int = 1) -> None:
    rc = lib().orc_dm_walk_fast(_p(t), n, h0, steps, seed, stream, rule, a, b, threads)
    assert rc == 0


def cftp_fast(tmax, tmin, n, seed, stream, first_sweeps, max_attempts, rule=1, a=0.7, b=1.0, threads: int = 1):
    tmax, tmin = _i32(tmax), _i32(tmin)
    out = np.zeros_like(tmax)
    used = C.c_long()
    att = lib().orc_dm_cftp_fast(_p(tmax), _p(tmin), n, seed, stream, first_sweeps, max_attempts, rule, a, b, threads,
                                 _p(out), C.addressof(used))
    return out, att, used.value


def tinymt_u32(seed, mat1, mat2, tmat, skip=0) -> int:
    return lib().orc_tinymt_u32(seed, mat1, mat2, tmat, skip)


def philox4x32_10(ctr, key):
    c = np.ascontiguousarray(np.asarray(ctr, np.uint32))
    k = np.ascontiguousarray(np.asarray(key, np.uint32))
    out = np.zeros(4, np.uint32)
    lib().orc_philox4x32_10(_p(c), _p(k), _p(out))
    return out


def tmt_seed_states(seed: int, count: int) -> np.ndarray:
    out = np.zeros((count, 4), np.uint32)
    lib().orc_tmt_seed_states(seed & 0xFFFFFFFF, count, _p(out))
    return out


# ---- lozenge ---------------------------------------------------------------------------
_LZ_SIG = {
    "orc_lz_almost_hex_domain": (C.c_int, [C.c_int, C.c_int, _P, _L]),
    "orc_lz_domain_to_vertices": (None, [_P, C.c_int, _P]),
    "orc_lz_max_tiling": (C.c_int, [_P, C.c_int, _P]),
    "orc_lz_min_tiling": (C.c_int, [_P, C.c_int, _P]),
    "orc_lz_heightfunc_to_tiling": (None, [_P, _P, C.c_int, _P]),
    "orc_lz_tiling_to_heightfunc": (None, [_P, _P, C.c_int, _P]),
    "orc_lz_tiling_to_domain": (None, [_P, C.c_int, _P]),
    "orc_lz_walk_tinymt": (C.c_int, [_P, C.c_int, _L, _L, _P, _L]),
    "orc_lz_walk_fast": (C.c_int, [_P, C.c_int, _L, _L, C.c_ulong, C.c_uint]),
    "orc_lz_walk_draws": (C.c_int, [_P, C.c_int, _P, _L, _L]),
    "orc_lz_cftp": (C.c_int, [_P, _P, C.c_int, _L, _L, C.c_int, C.c_int, C.c_int, C.c_uint, _P, _P]),
    "orc_lz_set_rule": (None, [C.c_int, C.c_double]),
}


def lz_lib() -> C.CDLL:
    h = lib()
    for name, (res, args) in _LZ_SIG.items():
        f = getattr(h, name)
        f.restype = res
        f.argtypes = args
    return h


def lz_almost_hex(n: int, m: int) -> np.ndarray:
    buf = np.zeros(2 * (2 * n + 9) ** 2, np.int32)
    rows = lz_lib().orc_lz_almost_hex_domain(n, m, _p(buf), buf.size)
    return buf[: 2 * rows * rows].copy()


def _tri(d) -> int:
    import math
    return math.isqrt(len(d) // 2)


def lz_extremal(d, which: str):
    d = _i32(d)
    m = _tri(d)
    out = np.zeros((m + 1) ** 2, np.int32)
    rc = getattr(lz_lib(), f"orc_lz_{which}_tiling")(_p(d), m, _p(out))
    return rc, out


def lz_tiling_to_heightfunc(t, d) -> np.ndarray:
    t, d = _i32(t), _i32(d)
    n = _side(t)
    out = np.zeros(n * n, np.int32)
    lz_lib().orc_lz_tiling_to_heightfunc(_p(t), _p(d), n, _p(out))
    return out


def lz_walk_tinymt(t: np.ndarray, n: int, steps: int, seed: int, params=None) -> None:
    p, cnt = _params(params)
    assert lz_lib().orc_lz_walk_tinymt(_p(t), n, steps, seed, _p(p), cnt) == 0


def lz_walk_draws(t: np.ndarray, n: int, draws: np.ndarray, steps: int, seed: int) -> None:
    """The reference's CUDA-path lozenge walk with its MTGP32 draws supplied (steps x n x n/3)."""
    d = np.ascontiguousarray(draws, np.float32)
    assert d.size == steps * n * (n // 3)
    assert lz_lib().orc_lz_walk_draws(_p(t), n, _p(d), steps, seed) == 0


def lz_walk_fast(t: np.ndarray, n: int, h0: int, steps: int, seed: int, stream: int = 0) -> None:
    assert lz_lib().orc_lz_walk_fast(_p(t), n, h0, steps, seed, stream) == 0


def lz_cftp(tmax, tmin, n, driver_seed, first, schedule, max_attempts, fast=False, stream=0):
    tmax, tmin = _i32(tmax), _i32(tmin)
    out = np.zeros_like(tmax)
    total = C.c_long()
    att = lz_lib().orc_lz_cftp(_p(tmax), _p(tmin), n, driver_seed, first, schedule, max_attempts, 1 if fast else 0,
                               stream, _p(out), C.addressof(total))
    return out, att, total.value


# ---- rectangle-triangle ----------------------------------------------------------------
_RT_SIG = {
    "orc_rt_hex": (C.c_int, [C.c_int, C.c_int, _P, _L]),
    "orc_rt_walk_tinymt": (C.c_int, [_P, C.c_int, _L, _L, _P, _P, _L]),
    "orc_rt_walk_fast": (C.c_int, [_P, C.c_int, _L, _L, C.c_ulong, C.c_uint, _P]),
    "orc_rt_walk_draws": (C.c_int, [_P, C.c_int, _P, _L, _L, _P]),
}
RT_UNIT_WEIGHTS = np.ones(9, np.float64)


def rt_lib() -> C.CDLL:
    h = lib()
    for name, (res, args) in _RT_SIG.items():
        f = getattr(h, name)
        f.restype = res
        f.argtypes = args
    return h


def rt_hex(n: int, top: bool) -> np.ndarray:
    buf = np.zeros((2 * n + 9) ** 2, np.int32)
    side = rt_lib().orc_rt_hex(n, 1 if top else 0, _p(buf), buf.size)
    assert side > 0
    return buf[: side * side].copy()


def _w9(weights) -> np.ndarray:
    return np.ascontiguousarray(RT_UNIT_WEIGHTS if weights is None else np.asarray(weights, np.float64))


def rt_walk_tinymt(t: np.ndarray, n: int, steps: int, seed: int, weights=None, params=None) -> None:
    w = _w9(weights)
    p, cnt = _params(params)
    assert rt_lib().orc_rt_walk_tinymt(_p(t), n, steps, seed, _p(w), _p(p), cnt) == 0


def rt_walk_fast(t: np.ndarray, n: int, h0: int, steps: int, seed: int, stream: int = 0, weights=None) -> None:
    w = _w9(weights)
    assert rt_lib().orc_rt_walk_fast(_p(t), n, h0, steps, seed, stream, _p(w)) == 0


# ---- six-vertex --------------------------------------------------------------------------
_SV_SIG = {
    "orc_sv_thresholds": (None, [C.c_double, C.c_double, C.c_double, _P]),
    "orc_sv_dwbc": (None, [C.c_int, C.c_int, _P]),
    "orc_sv_draw": (C.c_uint, [C.c_ulong, C.c_uint, _L, C.c_uint, C.c_uint]),
    "orc_sv_walk": (C.c_int, [_P, C.c_int, _L, _L, C.c_ulong, C.c_uint, C.c_double, C.c_double, C.c_double]),
    "orc_sv_cftp": (C.c_int, [_P, _P, C.c_int, C.c_ulong, C.c_uint, _L, C.c_int, C.c_double, C.c_double, C.c_double,
                              _P, _P]),
}


def sv_lib() -> C.CDLL:
    h = lib()
    for name, (res, args) in _SV_SIG.items():
        f = getattr(h, name)
        f.restype = res
        f.argtypes = args
    return h


def sv_thresholds(a, b, c) -> np.ndarray:
    out = np.zeros(9, np.uint32)
    sv_lib().orc_sv_thresholds(a, b, c, _p(out))
    return out


def sv_dwbc(n: int, top: bool) -> np.ndarray:
    out = np.zeros((n + 1) ** 2, np.int32)
    sv_lib().orc_sv_dwbc(n, 1 if top else 0, _p(out))
    return out


def sv_walk(h: np.ndarray, n: int, s0: int, count: int, seed: int, stream: int = 0, a=1.0, b=1.0, c=1.0) -> None:
    assert sv_lib().orc_sv_walk(_p(h), n, s0, count, seed, stream, a, b, c) == 0


def sv_cftp(hmax, hmin, n, seed, stream, first_sweeps, max_attempts, a=1.0, b=1.0, c=1.0):
    hmax, hmin = _i32(hmax), _i32(hmin)
    out = np.zeros_like(hmax)
    used = C.c_long()
    att = sv_lib().orc_sv_cftp(_p(hmax), _p(hmin), n, seed, stream, first_sweeps, max_attempts, a, b, c, _p(out),
                               C.addressof(used))
    return out, att, used.value


# ---- bibone (triangular-lattice dimers) -----------------------------------------------------
_TD_SIG = {
    "orc_td_icecream": (C.c_int, [C.c_int, C.c_int, _P, _L]),
    "orc_td_walk_tinymt": (C.c_int, [_P, C.c_int, _L, _L, _P, _L]),
    "orc_td_walk_fast": (C.c_int, [_P, C.c_int, _L, _L, C.c_ulong, C.c_uint]),
    "orc_td_walk_draws": (C.c_int, [_P, C.c_int, _P, _L, _L]),
    "orc_td_fast_step": (None, [C.c_ulong, C.c_uint, _L, _P]),
}


def td_lib() -> C.CDLL:
    h = lib()
    for name, (res, args) in _TD_SIG.items():
        f = getattr(h, name)
        f.restype = res
        f.argtypes = args
    return h


def td_icecream(n: int, m: int) -> np.ndarray:
    buf = np.zeros(4 * (n + 8) ** 2, np.int32)
    side = td_lib().orc_td_icecream(n, m, _p(buf), buf.size)
    assert side > 0
    return buf[: side * side].copy()


def td_walk_tinymt(t: np.ndarray, n_side: int, steps: int, seed: int, params=None) -> None:
    p, cnt = _params(params)
    assert td_lib().orc_td_walk_tinymt(_p(t), n_side, steps, seed, _p(p), cnt) == 0


def td_walk_draws(t: np.ndarray, n_side: int, draws: np.ndarray, steps: int, seed: int) -> None:
    """The reference's CUDA-path bibone walk with its MTGP32 draws supplied (steps x M x M)."""
    d = np.ascontiguousarray(draws, np.float32)
    assert d.size == steps * (n_side // 2) ** 2
    assert td_lib().orc_td_walk_draws(_p(t), n_side, _p(d), steps, seed) == 0


def td_walk_fast(t: np.ndarray, n_side: int, h0: int, steps: int, seed: int, stream: int = 0) -> None:
    assert td_lib().orc_td_walk_fast(_p(t), n_side, h0, steps, seed, stream) == 0


class lz_rule:
    """Context manager selecting the oracle's lozenge rotation rule (q = None: uniform)."""

    def __init__(self, q=None):
        self.q = q

    def __enter__(self):
        lz_lib().orc_lz_set_rule(0 if self.q is None else 1, 1.0 if self.q is None else float(self.q))
        return self

    def __exit__(self, *exc):
        lz_lib().orc_lz_set_rule(0, 1.0)


def rt_walk_draws(t: np.ndarray, n: int, draws: np.ndarray, steps: int, seed: int, weights=None) -> None:
    """The reference's CUDA-path rectangle-triangle walk with its MTGP32 draws supplied."""
    w = _w9(weights)
    d = np.ascontiguousarray(draws, np.float32)
    assert d.size == steps * n * (n // 3)
    assert rt_lib().orc_rt_walk_draws(_p(t), n, _p(d), steps, seed, _p(w)) == 0
