"""GB300-native random-tiling sampler: Python mirror of the reference's domino tiler API.

The reference exposes one C++ class per model (src/Domino/DominoTiler.h:46-131).  This
module keeps that shape - ``DominoTiler().Walk(t, steps, seed)``, ``DominoTiler.MaxTiling(d)``,
... - on top of the C ABI of ``librt_tilings.so`` (include/rt_tilings.h).  Domains, tilings
and height functions are flat int32 arrays of a square side, as the reference's
``std::vector<int>`` typedefs are (src/common/common.h:50-52).

Sweeps run on the GPU only; if the shared library is missing this module raises instead of
falling back to anything else.
"""
from __future__ import annotations

import ctypes as C
import math
import os
from dataclasses import dataclass
from pathlib import Path
from typing import Sequence

import numpy as np

_PKG = Path(__file__).resolve().parent
LIB_PATH = _PKG / "librt_tilings.so"

RT_MODEL_DOMINO, RT_MODEL_LOZENGE, RT_MODEL_RECTTRI, RT_MODEL_BIBONE, RT_MODEL_SIX_VERTEX = 0, 1, 2, 3, 4
RT_OK = 0
RT_ERR_INVALID_ARGUMENT = 1
RT_ERR_CUDA = 2
RT_ERR_NOT_TILEABLE = 3
RT_ERR_TIMEOUT = 4
RT_ERR_OUT_OF_MEMORY = 5
RT_ERR_NOT_COALESCED = 6
RT_ERR_BUFFER_TOO_SMALL = 7
RT_ERR_BUSY = 8

RNG_MODES = {"tinymt": 0, "fast": 1, "mtgp": 2}
RT_LOZENGE_UNIFORM, RT_LOZENGE_Q = 0, 1
DOMINO_RULES = {"plain": 0, "cftp": 1, "twoperiodic": 2, "cftp_twoperiodic": 3}


class RTError(RuntimeError):
    def __init__(self, status: int, message: str):
        super().__init__(f"{message} (status {status})")
        self.status = status


class _WalkOpts(C.Structure):
    _fields_ = [
        ("rng_mode", C.c_int32),
        ("rule", C.c_int32),
        ("weight_a", C.c_double),
        ("weight_b", C.c_double),
        ("tinymt_params", C.c_void_p),
        ("tinymt_params_count", C.c_int64),
        ("fast_stream", C.c_uint32),
        ("engine", C.c_int32),
        ("cuda_stream", C.c_void_p),
    ]


class CftpStats(C.Structure):
    _fields_ = [
        ("attempts", C.c_int32),
        ("total_steps", C.c_int64),
        ("final_steps", C.c_int64),
        ("flip_attempts", C.c_int64),
        ("seconds", C.c_double),
    ]

    def as_dict(self) -> dict:
        return {f: getattr(self, f) for f, _ in self._fields_}


class CftpInstance(C.Structure):
    _fields_ = [
        ("model", C.c_int32), ("n_side", C.c_int32), ("rule", C.c_int32), ("max_attempts", C.c_int32),
        ("weight_a", C.c_double), ("weight_b", C.c_double), ("seed", C.c_uint64), ("stream", C.c_uint32),
        ("pad", C.c_int32), ("first_steps", C.c_int64), ("tmax", C.c_void_p), ("tmin", C.c_void_p),
        ("out", C.c_void_p), ("attempts", C.c_int32), ("pad2", C.c_int32), ("final_steps", C.c_int64),
    ]


class BatchStats(C.Structure):
    _fields_ = [("instances", C.c_int32), ("coalesced", C.c_int32), ("ctas", C.c_int32), ("pad", C.c_int32),
                ("seconds", C.c_double), ("cluster_instances", C.c_int32), ("single_instances", C.c_int32)]


class ServerOpts(C.Structure):
    _fields_ = [("slots", C.c_int32), ("max_side", C.c_int32), ("memory_budget_bytes", C.c_int64),
                ("idle_seconds", C.c_double), ("cuda_stream", C.c_void_p)]


_P = C.c_void_p
_SIGNATURES = {
    "rt_walk_opts_default": (None, [_P]),
    "rt_status_string": (C.c_char_p, [C.c_int32]),
    "rt_last_error": (C.c_char_p, []),
    "rt_version": (C.c_char_p, []),
    "rt_domino_aztec_rectangle": (C.c_int32, [C.c_int32, _P, C.c_int32, _P, C.c_int64, _P]),
    "rt_domino_aztec_diamond": (C.c_int32, [C.c_int32, _P, C.c_int64, _P]),
    "rt_domino_rectangle": (C.c_int32, [C.c_int32, C.c_int32, _P, C.c_int64, _P]),
    "rt_domino_domain_to_vertices": (C.c_int32, [_P, C.c_int32, _P]),
    "rt_domino_max_tiling": (C.c_int32, [_P, C.c_int32, _P]),
    "rt_domino_min_tiling": (C.c_int32, [_P, C.c_int32, _P]),
    "rt_domino_extremal_tiling_device": (C.c_int32, [_P, C.c_int32, C.c_int32, _P, _P]),
    "rt_domino_tiling_to_heightfunc": (C.c_int32, [_P, _P, C.c_int32, _P]),
    "rt_domino_heightfunc_to_tiling": (C.c_int32, [_P, _P, C.c_int32, _P]),
    "rt_domino_tiling_to_domain": (C.c_int32, [_P, C.c_int32, _P]),
    "rt_domino_walk": (C.c_int32, [_P, C.c_int32, C.c_int64, C.c_int64, _P]),
    "rt_domino_walk_epochs": (C.c_int32, [_P, C.c_int32, _P, _P, C.c_int32, _P]),
    "rt_domino_cftp": (C.c_int32, [_P, _P, C.c_int32, C.c_int64, C.c_int64, C.c_int32, C.c_int32, _P, _P, _P]),
    "rt_dm_sampler_create": (C.c_int32, [C.c_int32, C.c_int32, _P, _P]),
    "rt_dm_sampler_destroy": (C.c_int32, [_P]),
    "rt_dm_sampler_load": (C.c_int32, [_P, C.c_int32, _P]),
    "rt_dm_sampler_store": (C.c_int32, [_P, C.c_int32, _P]),
    "rt_dm_sampler_copy_chain": (C.c_int32, [_P, C.c_int32, C.c_int32]),
    "rt_dm_sampler_set_active": (C.c_int32, [_P, C.c_int32]),
    "rt_dm_sampler_seed": (C.c_int32, [_P, C.c_uint32]),
    "rt_dm_sampler_run": (C.c_int32, [_P, _P, C.c_int64]),
    "rt_dm_sampler_run_fast": (C.c_int32, [_P, C.c_uint64, C.c_int64, C.c_int64]),
    "rt_dm_sampler_diff": (C.c_int32, [_P, C.c_int32, C.c_int32, _P]),
    "rt_dm_sampler_accumulate_edges": (C.c_int32, [_P, C.c_int32, _P]),
    "rt_dm_sampler_set_domain": (C.c_int32, [_P, _P, C.c_int32]),
    "rt_dm_sampler_accumulate_heights": (C.c_int32, [_P, C.c_int32, _P, _P]),
    "rt_domino_heightfunc_device": (C.c_int32, [_P, _P, C.c_int32, _P, _P]),
    "rt_domino_edge_indicators": (C.c_int32, [_P, C.c_int32, _P]),
    "rt_domino_aztec_edge_probs": (C.c_int32, [C.c_int32, C.c_double, C.c_double, _P, C.c_int64, _P]),
    "rt_dm_sampler_sync": (C.c_int32, [_P]),
    "rt_dm_sampler_stream": (C.c_void_p, [_P]),
    "rt_dm_sampler_interior_vertices": (C.c_int64, [_P]),
    "rt_dm_sampler_launches": (C.c_int64, [_P]),
    "rt_dm_sampler_engine_info": (C.c_int32, [_P, _P]),
    "rt_dm_sampler_set_launch": (C.c_int32, [_P, C.c_int32, C.c_int32, C.c_int32]),
    "rt_dm_sampler_launch_info": (C.c_int32, [_P, _P]),
    "rt_tune_load": (C.c_int32, [C.c_char_p]),
    "rt_tune_clear": (C.c_int32, []),
    "rt_tune_lookup": (C.c_int32, [C.c_int32, C.c_int32, C.c_int32, C.c_int32, _P]),
    "rt_dm_sampler_test_silent_band": (C.c_int32, [_P, C.c_int32, C.c_int64]),
    "rt_walk": (C.c_int32, [C.c_int32, _P, C.c_int32, C.c_int64, C.c_int64, _P, _P]),
    "rt_walk_epochs": (C.c_int32, [C.c_int32, _P, C.c_int32, _P, _P, C.c_int32, _P]),
    "rt_cftp": (C.c_int32, [C.c_int32, _P, _P, C.c_int32, C.c_int64, C.c_int64, C.c_int32, C.c_int32, _P, _P, _P,
                            _P]),
    "rt_domino_rule_table": (C.c_int32, [C.c_int32, C.c_int32, C.c_double, C.c_double, _P]),
    "rt_domino_mtgp_draws": (C.c_int32, [C.c_int32, C.c_int64, C.c_int64, _P]),
    "rt_lozenge_mtgp_draws": (C.c_int32, [C.c_int32, C.c_int64, C.c_int64, _P]),
    "rt_recttri_mtgp_draws": (C.c_int32, [C.c_int32, C.c_int64, C.c_int64, _P]),
    "rt_td_mtgp_draws": (C.c_int32, [C.c_int32, C.c_int64, C.c_int64, _P]),
    "rt_dm_sweep_noalloc": (C.c_int32, [_P, _P, C.c_int32, C.c_int32, _P, C.c_int64, C.c_uint64, C.c_int64, _P]),
    "rt_cftp_batch": (C.c_int32, [_P, C.c_int32, _P, _P]),
    "rt_server_create": (C.c_int32, [_P, _P]),
    "rt_server_submit": (C.c_int32, [_P, _P, _P]),
    "rt_server_poll": (C.c_int32, [_P, C.c_int64, _P]),
    "rt_server_wait": (C.c_int32, [_P, C.c_int64, C.c_double, _P]),
    "rt_server_destroy": (C.c_int32, [_P]),
    "rt_lozenge_almost_hex_domain": (C.c_int32, [C.c_int32, C.c_int32, _P, C.c_int64, _P]),
    "rt_lozenge_domain_to_vertices": (C.c_int32, [_P, C.c_int32, _P]),
    "rt_lozenge_max_tiling": (C.c_int32, [_P, C.c_int32, _P]),
    "rt_lozenge_min_tiling": (C.c_int32, [_P, C.c_int32, _P]),
    "rt_lozenge_heightfunc_to_tiling": (C.c_int32, [_P, _P, C.c_int32, _P]),
    "rt_lozenge_tiling_to_heightfunc": (C.c_int32, [_P, _P, C.c_int32, _P]),
    "rt_lozenge_tiling_to_domain": (C.c_int32, [_P, C.c_int32, _P]),
    "rt_lozenge_walk": (C.c_int32, [_P, C.c_int32, C.c_int64, C.c_int64, _P]),
    "rt_lozenge_cftp": (C.c_int32, [_P, _P, C.c_int32, C.c_int64, C.c_int64, C.c_int32, C.c_int32, _P, _P, _P]),
    "rt_recttri_hex_tiling": (C.c_int32, [C.c_int32, C.c_int32, _P, C.c_int64, _P]),
    "rt_recttri_from_lozenge": (C.c_int32, [_P, C.c_int32, _P, C.c_int32, _P]),
    "rt_recttri_walk": (C.c_int32, [_P, C.c_int32, C.c_int64, C.c_int64, _P, _P]),
    "rt_save_matrix": (C.c_int32, [_P, C.c_int64, C.c_int64, C.c_char_p]),
    "rt_save_matrix_square": (C.c_int32, [_P, C.c_int64, C.c_char_p]),
    "rt_load_matrix": (C.c_int32, [C.c_char_p, _P, C.c_int64, _P]),
    "rt_td_icecream_cone": (C.c_int32, [C.c_int32, C.c_int32, _P, C.c_int64, _P]),
    "rt_td_rhombus_brick": (C.c_int32, [C.c_int32, C.c_int32, _P, C.c_int64, _P]),
    "rt_td_dimers": (C.c_int32, [_P, C.c_int32, _P]),
    "rt_td_from_dimers": (C.c_int32, [_P, C.c_int32, _P]),
    "rt_td_walk": (C.c_int32, [_P, C.c_int32, C.c_int64, C.c_int64, _P, _P]),
    "rt_td_vertices": (C.c_int32, [_P, C.c_int32, _P]),
    "rt_td_test_butterfly": (C.c_int32, [C.c_int32, _P, C.c_int64, _P]),
    "rt_td_triangle_flips": (C.c_int32, [_P, C.c_int32, _P]),
    "rt_td_butterfly_flips": (C.c_int32, [_P, C.c_int32, _P]),
    "rt_td_domain": (C.c_int32, [_P, C.c_int32, _P]),
    "rt_td_dimer_indicator": (C.c_int32, [_P, C.c_int32, C.c_int32, _P]),
    "rt_sv_thresholds": (C.c_int32, [C.c_double, C.c_double, C.c_double, _P]),
    "rt_sv_dwbc_height": (C.c_int32, [C.c_int32, C.c_int32, _P]),
    "rt_sv_height_to_asm": (C.c_int32, [_P, C.c_int32, _P]),
    "rt_sv_asm_to_height": (C.c_int32, [_P, C.c_int32, _P]),
    "rt_sv_walk": (C.c_int32, [_P, C.c_int32, C.c_int64, C.c_int64, _P, _P, _P]),
    "rt_sv_cftp": (C.c_int32, [_P, _P, C.c_int32, C.c_int64, C.c_int64, C.c_int32, _P, _P, _P, _P]),
}

_lib_handle = None


def lib() -> C.CDLL:
    """Loads librt_tilings.so (built by ``randomtilingspublic_gb300.build``)."""
    global _lib_handle
    if _lib_handle is None:
        path = Path(os.environ.get("RT_TILINGS_LIB", LIB_PATH))
        if not path.exists():
            raise RuntimeError(
                f"{path} is missing: build it with `python -m randomtilingspublic_gb300.build` "
                "(the sampler has no non-CUDA implementation)")
        h = C.CDLL(str(path))
        for name, (res, args) in _SIGNATURES.items():
            fn = getattr(h, name)
            fn.restype = res
            fn.argtypes = args
        _lib_handle = h
    return _lib_handle


def _check(status: int) -> None:
    if status != RT_OK:
        msg = lib().rt_last_error().decode() or lib().rt_status_string(status).decode()
        raise RTError(status, msg)


def _i32(a) -> np.ndarray:
    return np.ascontiguousarray(np.asarray(a, dtype=np.int32).ravel())


def _ptr(a: np.ndarray) -> int:
    return a.ctypes.data


def side_of(a) -> int:
    n = math.isqrt(len(a))
    if n * n != len(a):
        raise ValueError("expected a square array")
    return n


def _write_back(dst, src: np.ndarray) -> None:
    """In-place update of the caller's tiling, as Walk(tiling&, ...) does."""
    if isinstance(dst, np.ndarray):
        dst.reshape(-1)[:] = src
    elif isinstance(dst, list):
        dst[:] = src.tolist()
    else:
        raise TypeError("tiling must be a numpy array or a list to be updated in place")


def read_tinymt_params(path: str | os.PathLike, count: int) -> np.ndarray:
    """Parameter file of TinyMTDC as LoadTinyMT reads it (src/TinyMT/file_reader.cpp:22-38,
    :142-158): lines starting with '#' are skipped; mat1, mat2, tmat are the hex fields after
    the 3rd, 4th and 5th comma.  Returns a (count, 3) uint32 array."""
    out = np.zeros((count, 3), dtype=np.uint32)
    k = 0
    with open(path) as f:
        for line in f:
            if k >= count:
                break
            if line.startswith("#") or not line.strip():
                continue
            fields = line.split(",")
            out[k] = [int(fields[3], 16), int(fields[4], 16), int(fields[5], 16)]
            k += 1
    if k < count:
        raise ValueError(f"{path} holds {k} parameter sets, {count} needed")
    return out


class _TinyMTTable:
    """LoadTinyMT(params, size) of every reference tiler (DominoTiler.cpp:235-237,
    LozengeTiler.cpp:161-164, RectTriangleTiler.cpp:22-25, TriangleDimerTiler.cpp:24-27): the
    per-generator TinyMT parameters of its OpenCL path, triple k for generator k."""

    _params: np.ndarray | None = None

    def LoadTinyMT(self, params, size: int | None = None) -> None:
        """Loads per-generator TinyMT parameters: a TinyMTDC file path (with ``size`` sets)
        or an (n, 3) array of (mat1, mat2, tmat)."""
        if isinstance(params, (str, os.PathLike)):
            if size is None:
                raise ValueError("size is required with a parameter file")
            self._params = read_tinymt_params(params, size)
        else:
            self._params = np.ascontiguousarray(np.asarray(params, dtype=np.uint32).reshape(-1, 3))

    def _apply_params(self, o: "_WalkOpts") -> None:
        if self._params is not None:
            o.tinymt_params = self._params.ctypes.data
            o.tinymt_params_count = self._params.shape[0]


class DominoTiler(_TinyMTTable):
    """Domino tilings (src/Domino/DominoTiler.h:46-131).

    ``rule`` selects what the reference selects by compiling one of its kernel files:
    'plain' (dominokernel), 'cftp' (dominokernelCFTP), 'twoperiodic', 'cftp_twoperiodic';
    ``a``, ``b`` are the two-periodic weights the reference hard-codes (0.7, 1.0).
    ``rng`` is 'tinymt' (bit-exact with the reference's OpenCL path), 'mtgp' (cuRAND MTGP32
    as the reference's CUDA path draws it; also selected by LoadMTGP) or 'fast' (Philox).
    ``engine``: 0 automatic, 1 per-half-sweep kernels, 2 the run kernel, 3 k_persist, 4 the
    bit-plane kernel; every engine gives the same tilings.
    """

    def __init__(self, rule: str = "plain", rng: str = "tinymt", a: float = 0.7, b: float = 1.0,
                 fast_stream: int = 0, engine: int = 0):
        self.rule = rule
        self.rng = rng
        self.a = float(a)
        self.b = float(b)
        self.fast_stream = int(fast_stream)
        self.engine = int(engine)
        self._params: np.ndarray | None = None

    # -- reference: LoadTinyMT(params, size) (the mixin) / LoadMTGP() -----------------------
    def LoadMTGP(self) -> None:
        """DominoTiler::LoadMTGP (DominoTiler.cpp:239-242): walks draw from cuRAND MTGP32, one
        generator per 8 x 8 block of sites seeded seed + block, as the reference's CUDA build."""
        self.rng = "mtgp"

    def opts(self, cuda_stream: int | None = None) -> _WalkOpts:
        o = _WalkOpts()
        lib().rt_walk_opts_default(C.byref(o))
        o.rng_mode = RNG_MODES[self.rng]
        o.rule = DOMINO_RULES[self.rule]
        o.weight_a = self.a
        o.weight_b = self.b
        o.fast_stream = self.fast_stream
        o.engine = self.engine
        self._apply_params(o)
        if cuda_stream:
            o.cuda_stream = cuda_stream
        return o

    # -- reference: Walk(t, steps, seed) and Walk(t, vector steps, vector seeds) -------------
    def Walk(self, t, steps, seeds) -> None:
        tt = _i32(t)
        n = side_of(tt)
        o = self.opts()
        if isinstance(steps, (list, tuple, np.ndarray)):
            st = np.ascontiguousarray(np.asarray(steps, dtype=np.int64))
            sd = np.ascontiguousarray(np.asarray(seeds, dtype=np.int64))
            if st.shape != sd.shape:
                raise ValueError("steps and seeds must have the same length")
            _check(lib().rt_domino_walk_epochs(_ptr(tt), n, _ptr(st), _ptr(sd), len(st), C.byref(o)))
        else:
            _check(lib().rt_domino_walk(_ptr(tt), n, int(steps), int(seeds), C.byref(o)))
        _write_back(t, tt)

    def cftp(self, tmax, tmin, driver_seed: int, first_steps: int = 128, schedule: int = 0,
             max_attempts: int = 20):
        """Coupling from the past (Examples/AztecDiamondCftpEx.cpp:51-77); returns
        (tiling, stats dict).  Needs rule 'cftp' or 'cftp_twoperiodic'."""
        a, b = _i32(tmax), _i32(tmin)
        n = side_of(a)
        out = np.zeros_like(a)
        stats = CftpStats()
        o = self.opts()
        _check(lib().rt_domino_cftp(_ptr(a), _ptr(b), n, int(driver_seed), int(first_steps), int(schedule),
                                    int(max_attempts), C.byref(o), _ptr(out), C.byref(stats)))
        return out, stats.as_dict()

    # -- static utilities (DominoTiler.cpp:249-631) -----------------------------------------
    @staticmethod
    def AztecRectangle(n: int, remove: Sequence[int] = ()) -> np.ndarray:
        rm = _i32(list(remove)) if len(remove) else None
        side = C.c_int32()
        m = 2 * n - len(remove) + 5
        buf = np.zeros(m * m, dtype=np.int32)
        _check(lib().rt_domino_aztec_rectangle(n, _ptr(rm) if rm is not None else None, len(remove), _ptr(buf),
                                               buf.size, C.byref(side)))
        return buf[: side.value * side.value].copy()

    @staticmethod
    def AztecDiamond(n: int) -> np.ndarray:
        return DominoTiler.AztecRectangle(n, ())

    @staticmethod
    def Rectangle(rows: int, cols: int) -> np.ndarray:
        m = max(rows, cols) + 5
        buf = np.zeros(m * m, dtype=np.int32)
        side = C.c_int32()
        _check(lib().rt_domino_rectangle(rows, cols, _ptr(buf), buf.size, C.byref(side)))
        return buf[: side.value * side.value].copy()

    @staticmethod
    def DomainToVertices(d) -> np.ndarray:
        dd = _i32(d)
        m = side_of(dd)
        out = np.zeros((m + 1) ** 2, dtype=np.int32)
        _check(lib().rt_domino_domain_to_vertices(_ptr(dd), m, _ptr(out)))
        return out

    @staticmethod
    def MaxTiling(d) -> np.ndarray:
        dd = _i32(d)
        m = side_of(dd)
        out = np.zeros((m + 1) ** 2, dtype=np.int32)
        _check(lib().rt_domino_max_tiling(_ptr(dd), m, _ptr(out)))
        return out

    @staticmethod
    def MinTiling(d) -> np.ndarray:
        dd = _i32(d)
        m = side_of(dd)
        out = np.zeros((m + 1) ** 2, dtype=np.int32)
        _check(lib().rt_domino_min_tiling(_ptr(dd), m, _ptr(out)))
        return out

    @staticmethod
    def TilingToHeightfuncDevice(t, d) -> np.ndarray:
        """TilingToHeightfunc computed on the GPU (rt_domino_heightfunc_device)."""
        tt, dd = _i32(t), _i32(d)
        n = side_of(tt)
        out = np.zeros(n * n, dtype=np.int32)
        _check(lib().rt_domino_heightfunc_device(_ptr(tt), _ptr(dd), n, _ptr(out), None))
        return out

    @staticmethod
    def ExtremalTilingDevice(d, top: bool) -> np.ndarray:
        """MaxTiling (top) / MinTiling computed on the GPU (rt_domino_extremal_tiling_device)."""
        dd = _i32(d)
        m = side_of(dd)
        out = np.zeros((m + 1) ** 2, dtype=np.int32)
        _check(lib().rt_domino_extremal_tiling_device(_ptr(dd), m, 1 if top else 0, _ptr(out), None))
        return out

    @staticmethod
    def TilingToHeightfunc(t, d) -> np.ndarray:
        tt, dd = _i32(t), _i32(d)
        n = side_of(tt)
        out = np.zeros(n * n, dtype=np.int32)
        _check(lib().rt_domino_tiling_to_heightfunc(_ptr(tt), _ptr(dd), n, _ptr(out)))
        return out

    @staticmethod
    def HeightfuncToTiling(hf, d) -> np.ndarray:
        hh, dd = _i32(hf), _i32(d)
        n = side_of(hh)
        out = np.zeros(n * n, dtype=np.int32)
        _check(lib().rt_domino_heightfunc_to_tiling(_ptr(hh), _ptr(dd), n, _ptr(out)))
        return out

    @staticmethod
    def TilingToDomain(t) -> np.ndarray:
        tt = _i32(t)
        n = side_of(tt)
        out = np.zeros((n - 1) ** 2, dtype=np.int32)
        _check(lib().rt_domino_tiling_to_domain(_ptr(tt), n, _ptr(out)))
        return out


def _tri_side(d) -> int:
    m = math.isqrt(len(d) // 2)
    if 2 * m * m != len(d):
        raise ValueError("expected an M x 2M triangle array")
    return m


class LozengeTiler(_TinyMTTable):
    """Lozenge tilings (src/Lozenge/LozengeTiler.h:46-92).  ``rng`` is 'tinymt' (bit-exact
    with the reference's OpenCL path), 'mtgp' (its CUDA path's cuRAND MTGP32 draws, uniform
    rule; also selected by LoadMTGP) or 'fast'."""

    def __init__(self, rng: str = "tinymt", fast_stream: int = 0, q: float | None = None, engine: int = 0):
        """q: None for the reference's uniform rotation (lozengekernel.cl), else the q^volume
        rotation of qlozengekernel.cl (down-move rescaling corrected).  engine: 0 automatic (the
        resident band kernel where it holds the size), 1 the per-step kernels, 2 the resident
        band kernel (an error where it does not hold the size); every engine gives the same
        tilings."""
        self.rng = rng
        self.fast_stream = int(fast_stream)
        self.q = q
        self.engine = int(engine)

    def LoadMTGP(self) -> None:
        """LozengeTiler::LoadMTGP: walks draw from cuRAND MTGP32 block generators, as the
        reference's CUDA build (LozengeTiler.cpp:71-80)."""
        self.rng = "mtgp"

    def opts(self) -> _WalkOpts:
        o = _WalkOpts()
        lib().rt_walk_opts_default(C.byref(o))
        o.rng_mode = RNG_MODES[self.rng]
        o.fast_stream = self.fast_stream
        o.engine = self.engine
        if self.q is not None:
            o.rule = RT_LOZENGE_Q
            o.weight_a = float(self.q)
        else:
            o.rule = RT_LOZENGE_UNIFORM
        self._apply_params(o)
        return o

    def Walk(self, t, steps: int, seed: int) -> None:
        tt = _i32(t)
        o = self.opts()
        _check(lib().rt_lozenge_walk(_ptr(tt), side_of(tt), int(steps), int(seed), C.byref(o)))
        _write_back(t, tt)

    def cftp(self, tmax, tmin, driver_seed: int, first_steps: int = 128, schedule: int = 0, max_attempts: int = 20):
        a, b = _i32(tmax), _i32(tmin)
        out = np.zeros_like(a)
        stats = CftpStats()
        o = self.opts()
        _check(lib().rt_lozenge_cftp(_ptr(a), _ptr(b), side_of(a), int(driver_seed), int(first_steps), int(schedule),
                                     int(max_attempts), C.byref(o), _ptr(out), C.byref(stats)))
        return out, stats.as_dict()

    @staticmethod
    def AlmostHexDomain(n: int, m: int) -> np.ndarray:
        rows = C.c_int32()
        r = 2 * n + 8
        buf = np.zeros(2 * r * r, np.int32)
        _check(lib().rt_lozenge_almost_hex_domain(n, m, _ptr(buf), buf.size, C.byref(rows)))
        return buf[: 2 * rows.value * rows.value].copy()

    @staticmethod
    def Hexagon(n: int) -> np.ndarray:
        """The a = b = c = n hexagon (declared at LozengeTiler.h:77; AlmostHexDomain(n, 0))."""
        return LozengeTiler.AlmostHexDomain(n, 0)

    @staticmethod
    def DomainToVertices(d) -> np.ndarray:
        dd = _i32(d)
        m = _tri_side(dd)
        out = np.zeros((m + 1) ** 2, np.int32)
        _check(lib().rt_lozenge_domain_to_vertices(_ptr(dd), m, _ptr(out)))
        return out

    @staticmethod
    def MaxTiling(d) -> np.ndarray:
        dd = _i32(d)
        m = _tri_side(dd)
        out = np.zeros((m + 1) ** 2, np.int32)
        _check(lib().rt_lozenge_max_tiling(_ptr(dd), m, _ptr(out)))
        return out

    @staticmethod
    def MinTiling(d) -> np.ndarray:
        dd = _i32(d)
        m = _tri_side(dd)
        out = np.zeros((m + 1) ** 2, np.int32)
        _check(lib().rt_lozenge_min_tiling(_ptr(dd), m, _ptr(out)))
        return out

    @staticmethod
    def TilingToHeightfunc(t, d) -> np.ndarray:
        tt, dd = _i32(t), _i32(d)
        n = side_of(tt)
        out = np.zeros(n * n, np.int32)
        _check(lib().rt_lozenge_tiling_to_heightfunc(_ptr(tt), _ptr(dd), n, _ptr(out)))
        return out

    @staticmethod
    def HeightfuncToTiling(hf, d) -> np.ndarray:
        hh, dd = _i32(hf), _i32(d)
        n = side_of(hh)
        out = np.zeros(n * n, np.int32)
        _check(lib().rt_lozenge_heightfunc_to_tiling(_ptr(hh), _ptr(dd), n, _ptr(out)))
        return out

    @staticmethod
    def TilingToDomain(t) -> np.ndarray:
        tt = _i32(t)
        n = side_of(tt)
        out = np.zeros(2 * (n - 1) ** 2, np.int32)
        _check(lib().rt_lozenge_tiling_to_domain(_ptr(tt), n, _ptr(out)))
        return out


class RectTriangleTiler(_TinyMTTable):
    """Rectangle-triangle tilings (src/RectTriangle/RectTriangleTiler.h:32-86).  ``weights``
    holds the nine tile weights {wt1, wt2, wt3, wm1, wm2, wm3, wr1, wr2, wr3}
    (recttrianglekernel.cl:3-11; all 1 by default, the reference's values).  ``rng`` is
    'tinymt' (bit-exact with the reference's OpenCL path), 'mtgp' (its CUDA path's cuRAND
    MTGP32 draws; also selected by LoadMTGP) or 'fast'."""

    def __init__(self, rng: str = "tinymt", fast_stream: int = 0, weights=None):
        self.rng = rng
        self.fast_stream = int(fast_stream)
        self.weights = None if weights is None else np.ascontiguousarray(weights, np.float64)
        if self.weights is not None and self.weights.shape != (9,):
            raise ValueError("weights: nine values {wt1, wt2, wt3, wm1, wm2, wm3, wr1, wr2, wr3}")

    def LoadMTGP(self) -> None:
        """RectTriangleTiler::LoadMTGP (RectTriangleTiler.cpp:27-30): walks draw from cuRAND
        MTGP32 block generators, as the reference's CUDA build."""
        self.rng = "mtgp"

    def opts(self) -> _WalkOpts:
        o = _WalkOpts()
        lib().rt_walk_opts_default(C.byref(o))
        o.rng_mode = RNG_MODES[self.rng]
        o.fast_stream = self.fast_stream
        self._apply_params(o)
        return o

    def Walk(self, t, steps: int, seed: int) -> None:
        tt = _i32(t)
        o = self.opts()
        w = None if self.weights is None else self.weights.ctypes.data
        _check(lib().rt_recttri_walk(_ptr(tt), side_of(tt), int(steps), int(seed), w, C.byref(o)))
        _write_back(t, tt)

    @staticmethod
    def _hex(n: int, top: int) -> np.ndarray:
        side = C.c_int32()
        s = 2 * n + 9
        buf = np.zeros(s * s, np.int32)
        _check(lib().rt_recttri_hex_tiling(int(n), top, _ptr(buf), buf.size, C.byref(side)))
        return buf[: side.value * side.value].copy()

    @staticmethod
    def maxHex(n: int) -> np.ndarray:
        return RectTriangleTiler._hex(n, 1)

    @staticmethod
    def minHex(n: int) -> np.ndarray:
        return RectTriangleTiler._hex(n, 0)

    @staticmethod
    def slopeHex(n: int) -> np.ndarray:
        return RectTriangleTiler._hex(n, 2)

    @staticmethod
    def LozengeToRectTriangle(t, d) -> np.ndarray:
        tt, dd = _i32(t), _i32(d)
        n = side_of(tt)
        out = np.zeros(n * n, np.int32)
        _check(lib().rt_recttri_from_lozenge(_ptr(tt), n, _ptr(dd), _tri_side(dd), _ptr(out)))
        return out


class TriangleDimerTiler(_TinyMTTable):
    """Bibone tilings, i.e. dimer coverings of the triangular lattice
    (src/TriangleDimer/TriangleDimerTiler.h:84-216).  ``rng`` is 'tinymt' (bit-exact with the
    reference's OpenCL path), 'mtgp' (its CUDA path's cuRAND MTGP32 draws; also selected by
    LoadMTGP) or 'fast'."""

    def __init__(self, rng: str = "tinymt", fast_stream: int = 0):
        self.rng = rng
        self.fast_stream = int(fast_stream)

    def LoadMTGP(self) -> None:
        """TriangleDimerTiler::LoadMTGP (TriangleDimerTiler.cpp:29-32): walks draw from cuRAND
        MTGP32 block generators, as the reference's CUDA build."""
        self.rng = "mtgp"

    def opts(self) -> _WalkOpts:
        o = _WalkOpts()
        lib().rt_walk_opts_default(C.byref(o))
        o.rng_mode = RNG_MODES[self.rng]
        o.fast_stream = self.fast_stream
        self._apply_params(o)
        return o

    def Walk(self, t, steps: int, seed: int) -> dict:
        tt = _i32(t)
        o, st = self.opts(), CftpStats()
        _check(lib().rt_td_walk(_ptr(tt), side_of(tt), int(steps), int(seed), C.byref(o), C.byref(st)))
        _write_back(t, tt)
        return st.as_dict()

    @staticmethod
    def IceCreamCone(n: int, m: int) -> np.ndarray:
        side = C.c_int32()
        s = 2 * (n + 4)
        buf = np.zeros(s * s, np.int32)
        _check(lib().rt_td_icecream_cone(int(n), int(m), _ptr(buf), buf.size, C.byref(side)))
        return buf[: side.value * side.value].copy()

    @staticmethod
    def RhombusBrick(rows: int, cols: int) -> np.ndarray:
        side = C.c_int32()
        s = 2 * (max(rows, cols) + 6)
        buf = np.zeros(s * s, np.int32)
        _check(lib().rt_td_rhombus_brick(int(rows), int(cols), _ptr(buf), buf.size, C.byref(side)))
        return buf[: side.value * side.value].copy()

    @staticmethod
    def Dimers(t) -> np.ndarray:
        """Dimer bytes ((N/2) x (N/2)): bit 1 (a,b)-(a,b+1), 2 (a,b)-(a-1,b), 4 (a,b)-(a-1,b+1)."""
        tt = _i32(t)
        n = side_of(tt)
        out = np.zeros((n // 2) ** 2, np.uint8)
        _check(lib().rt_td_dimers(_ptr(tt), n, _ptr(out)))
        return out

    @staticmethod
    def TestButterfly(type_: int) -> np.ndarray:
        side = C.c_int32()
        buf = np.zeros(16 * 16, np.int32)
        _check(lib().rt_td_test_butterfly(int(type_), _ptr(buf), buf.size, C.byref(side)))
        return buf

    @staticmethod
    def TilingToTriangleFlips(t) -> np.ndarray:
        tt = _i32(t)
        n = side_of(tt)
        out = np.zeros((n // 2) * n, np.int32)
        _check(lib().rt_td_triangle_flips(_ptr(tt), n, _ptr(out)))
        return out

    @staticmethod
    def TilingToButterflyFlips(t) -> np.ndarray:
        tt = _i32(t)
        n = side_of(tt)
        out = np.zeros(n * n, np.int32)
        _check(lib().rt_td_butterfly_flips(_ptr(tt), n, _ptr(out)))
        return out

    @staticmethod
    def TilingToVertices(t) -> np.ndarray:
        tt = _i32(t)
        n = side_of(tt)
        out = np.zeros((n // 2 + 1) ** 2, np.int32)
        _check(lib().rt_td_vertices(_ptr(tt), n, _ptr(out)))
        return out

    @staticmethod
    def TilingToDomain(t) -> np.ndarray:
        tt = _i32(t)
        n = side_of(tt)
        out = np.zeros((n // 2) * n, np.int32)
        _check(lib().rt_td_domain(_ptr(tt), n, _ptr(out)))
        return out

    @staticmethod
    def DimerIndicator(t, c: int) -> np.ndarray:
        tt = _i32(t)
        n = side_of(tt)
        out = np.zeros((n // 2) ** 2, np.int32)
        _check(lib().rt_td_dimer_indicator(_ptr(tt), n, int(c), _ptr(out)))
        return out

    @staticmethod
    def FromDimers(d, n_side: int) -> np.ndarray:
        dd = np.ascontiguousarray(np.asarray(d, np.uint8).ravel())
        out = np.zeros(n_side * n_side, np.int32)
        _check(lib().rt_td_from_dimers(_ptr(dd), int(n_side), _ptr(out)))
        return out


class SixVertexTiler:
    """Six-vertex model on an n x n grid (no counterpart in the reference; shaped like its
    per-model classes).  State: the (n+1) x (n+1) int32 height function; weights a, b, c;
    fast (Philox) random mode only, ``fast_stream`` selects an independent stream.  ``engine``:
    0 automatic, 1 one kernel per sub-sweep, 2 the cluster-resident kernel."""

    def __init__(self, a: float = 1.0, b: float = 1.0, c: float = 1.0, fast_stream: int = 0, engine: int = 0):
        self.abc = np.array([a, b, c], np.float64)
        self.fast_stream = int(fast_stream)
        self.engine = int(engine)

    def opts(self) -> _WalkOpts:
        o = _WalkOpts()
        lib().rt_walk_opts_default(C.byref(o))
        o.rng_mode = RNG_MODES["fast"]
        o.fast_stream = self.fast_stream
        o.engine = self.engine
        return o

    def Walk(self, h, sweeps: int, seed: int) -> dict:
        hh = _i32(h)
        o, st = self.opts(), CftpStats()
        _check(lib().rt_sv_walk(_ptr(hh), side_of(hh) - 1, int(sweeps), int(seed), self.abc.ctypes.data, C.byref(o),
                                C.byref(st)))
        _write_back(h, hh)
        return st.as_dict()

    def cftp(self, hmax, hmin, seed: int, first_sweeps: int = 16, max_attempts: int = 20):
        a, b = _i32(hmax), _i32(hmin)
        out = np.zeros_like(a)
        o, st = self.opts(), CftpStats()
        _check(lib().rt_sv_cftp(_ptr(a), _ptr(b), side_of(a) - 1, int(seed), int(first_sweeps), int(max_attempts),
                                self.abc.ctypes.data, C.byref(o), _ptr(out), C.byref(st)))
        return out, st.as_dict()

    @staticmethod
    def Thresholds(a: float, b: float, c: float) -> np.ndarray:
        out = np.zeros(9, np.uint32)
        _check(lib().rt_sv_thresholds(float(a), float(b), float(c), _ptr(out)))
        return out

    @staticmethod
    def MaxHeight(n: int) -> np.ndarray:
        """Domain-wall boundary, maximal height function min(x + y, 2n - x - y)."""
        out = np.zeros((n + 1) ** 2, np.int32)
        _check(lib().rt_sv_dwbc_height(int(n), 1, _ptr(out)))
        return out

    @staticmethod
    def MinHeight(n: int) -> np.ndarray:
        """Domain-wall boundary, minimal height function |x - y|."""
        out = np.zeros((n + 1) ** 2, np.int32)
        _check(lib().rt_sv_dwbc_height(int(n), 0, _ptr(out)))
        return out

    @staticmethod
    def HeightToASM(h) -> np.ndarray:
        hh = _i32(h)
        n = side_of(hh) - 1
        out = np.zeros(n * n, np.int32)
        _check(lib().rt_sv_height_to_asm(_ptr(hh), n, _ptr(out)))
        return out

    @staticmethod
    def ASMToHeight(a) -> np.ndarray:
        aa = _i32(a)
        n = side_of(aa)
        out = np.zeros((n + 1) ** 2, np.int32)
        _check(lib().rt_sv_asm_to_height(_ptr(aa), n, _ptr(out)))
        return out


class DominoSampler:
    """Device-resident coupled chains (rt_dm_sampler_*): the chains stay in HBM between
    calls; all chains share one random stream."""

    def __init__(self, n_side: int, n_chains: int, tiler: DominoTiler, cuda_stream: int | None = None):
        self._tiler = tiler
        self._o = tiler.opts(cuda_stream)
        h = C.c_void_p()
        _check(lib().rt_dm_sampler_create(n_side, n_chains, C.byref(self._o), C.byref(h)))
        self.h = h
        self.n = n_side

    def close(self) -> None:
        if self.h:
            lib().rt_dm_sampler_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def load(self, chain: int, t) -> None:
        tt = _i32(t)
        _check(lib().rt_dm_sampler_load(self.h, chain, _ptr(tt)))

    def store(self, chain: int) -> np.ndarray:
        out = np.zeros(self.n * self.n, dtype=np.int32)
        _check(lib().rt_dm_sampler_store(self.h, chain, _ptr(out)))
        return out

    def set_active(self, k: int) -> None:
        _check(lib().rt_dm_sampler_set_active(self.h, k))

    def copy_chain(self, dst: int, src: int) -> None:
        _check(lib().rt_dm_sampler_copy_chain(self.h, dst, src))

    def seed(self, seed: int) -> None:
        _check(lib().rt_dm_sampler_seed(self.h, seed & 0xFFFFFFFF))

    def run(self, colours: np.ndarray) -> None:
        c = np.ascontiguousarray(np.asarray(colours, dtype=np.uint8))
        _check(lib().rt_dm_sampler_run(self.h, _ptr(c), c.size))

    def run_fast(self, seed: int, h0: int, steps: int) -> None:
        _check(lib().rt_dm_sampler_run_fast(self.h, seed, h0, steps))

    def set_domain(self, d) -> None:
        """The (N-1) x (N-1) face array the chains tile (for accumulate_heights)."""
        self._domain = _i32(d)
        _check(lib().rt_dm_sampler_set_domain(self.h, _ptr(self._domain), side_of(self._domain)))

    def accumulate_heights(self, chain: int, sums_device_ptr: int = 0, heights_device_ptr: int = 0) -> None:
        """Adds the chain's height function to int64 device sums (N^2) and/or writes it to an
        int32 device array, on the sampler's stream."""
        _check(lib().rt_dm_sampler_accumulate_heights(self.h, int(chain), C.c_void_p(sums_device_ptr or None),
                                                      C.c_void_p(heights_device_ptr or None)))

    def accumulate_edges(self, chain: int, counts_device_ptr: int) -> None:
        """Adds chain's edge-placement indicators to a device array of 2 N^2 uint32 counters
        (e.g. a torch.int32 tensor's data_ptr()), on the sampler's stream."""
        _check(lib().rt_dm_sampler_accumulate_edges(self.h, int(chain), C.c_void_p(counts_device_ptr)))

    def diff(self, a: int, b: int) -> int:
        n = C.c_int64()
        _check(lib().rt_dm_sampler_diff(self.h, a, b, C.byref(n)))
        return n.value

    def sync(self) -> None:
        _check(lib().rt_dm_sampler_sync(self.h))

    @property
    def stream(self) -> int:
        return lib().rt_dm_sampler_stream(self.h) or 0

    @property
    def interior_vertices(self) -> int:
        return lib().rt_dm_sampler_interior_vertices(self.h)

    @property
    def launches(self) -> int:
        return lib().rt_dm_sampler_launches(self.h)

    def engine_info(self) -> dict:
        out = np.zeros(6, np.int64)
        _check(lib().rt_dm_sampler_launch_info(self.h, _ptr(out)))
        return {"engine": int(out[0]), "units": int(out[1]), "bands": int(out[2]), "units_per_thread": int(out[3]),
                "threads": int(out[4]), "tuned": bool(out[5])}

    def set_launch(self, engine: int = 0, bands: int = 0, threads: int = 0) -> None:
        """Launch shape of the next runs (rt_dm_sampler_set_launch): engine 0 automatic, 1
        per-half-sweep kernels, 2 the run kernel, 3 k_persist, 4 the bit-plane kernel; bands
        (run and bit-plane kernels) and threads per band (run kernel; 0: defaults).  Results
        do not depend on it."""
        _check(lib().rt_dm_sampler_set_launch(self.h, int(engine), int(bands), int(threads)))


def cftp_batch(jobs, cuda_stream: int | None = None):
    """Batched fast-mode CFTP (rt_cftp_batch).  jobs: dicts with model ('domino' or
    'lozenge'), tmax, tmin, seed, stream and optional rule, a, b, first_steps, max_attempts.
    Returns (samples, per-job attempts, stats dict)."""
    n = len(jobs)
    arr = (CftpInstance * n)()
    keep = []
    outs = []
    for k, j in enumerate(jobs):
        tmax, tmin = _i32(j["tmax"]), _i32(j["tmin"])
        out = np.empty_like(tmax)  # every cell is written by the call
        keep += [tmax, tmin]
        outs.append(out)
        x = arr[k]
        x.model = 0 if j["model"] == "domino" else 1
        x.n_side = side_of(tmax)
        x.rule = DOMINO_RULES[j.get("rule", "cftp")]
        x.max_attempts = int(j.get("max_attempts", 20))
        x.weight_a, x.weight_b = float(j.get("a", 1.0)), float(j.get("b", 1.0))
        x.seed, x.stream = int(j["seed"]), int(j["stream"])
        x.first_steps = int(j.get("first_steps", 8))
        x.tmax, x.tmin, x.out = _ptr(tmax), _ptr(tmin), _ptr(out)
    stats = BatchStats()
    st = lib().rt_cftp_batch(arr, n, cuda_stream, C.byref(stats))
    if st not in (RT_OK, RT_ERR_NOT_COALESCED):
        _check(st)
    attempts = [arr[k].attempts for k in range(n)]
    return outs, attempts, {f: getattr(stats, f) for f, _ in BatchStats._fields_ if f != "pad"}


def _instance(job) -> tuple:
    tmax, tmin = _i32(job["tmax"]), _i32(job["tmin"])
    x = CftpInstance()
    x.model = 0 if job["model"] == "domino" else 1
    x.n_side = side_of(tmax)
    x.rule = DOMINO_RULES[job.get("rule", "cftp")]
    x.max_attempts = int(job.get("max_attempts", 20))
    x.weight_a, x.weight_b = float(job.get("a", 1.0)), float(job.get("b", 1.0))
    x.seed, x.stream = int(job["seed"]), int(job["stream"])
    x.first_steps = int(job.get("first_steps", 8))
    x.tmax, x.tmin = _ptr(tmax), _ptr(tmin)
    return x, (tmax, tmin)


class Server:
    """Continuous-batching CFTP server (rt_server_*): submit requests as they arrive, collect
    each result when done."""

    def __init__(self, slots: int = 4096, max_side: int = 130, memory_budget_bytes: int = 120 << 30,
                 idle_seconds: float = 0.25):
        o = ServerOpts(slots, max_side, memory_budget_bytes, idle_seconds, None)
        h = C.c_void_p()
        _check(lib().rt_server_create(C.byref(o), C.byref(h)))
        self.h = h
        self._side = {}

    def submit(self, job) -> int:
        x, keep = _instance(job)
        t = C.c_int64()
        _check(lib().rt_server_submit(self.h, C.byref(x), C.byref(t)))
        self._side[t.value] = side_of(keep[0])
        return t.value

    def poll(self, ticket: int) -> bool:
        d = C.c_int32()
        _check(lib().rt_server_poll(self.h, ticket, C.byref(d)))
        return bool(d.value)

    def wait(self, ticket: int, timeout: float = 60.0):
        n = self._side.pop(ticket)
        out = np.zeros(n * n, np.int32)
        x = CftpInstance()
        x.out = _ptr(out)
        st = lib().rt_server_wait(self.h, ticket, timeout, C.byref(x))
        if st not in (RT_OK, RT_ERR_NOT_COALESCED):
            _check(st)
        return out, x.attempts, x.final_steps

    def close(self) -> None:
        if self.h:
            lib().rt_server_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def mt19937_colours(seed: int, steps: int, skip: int = 0) -> np.ndarray:
    """Colour stream of the reference's host loop: mt19937(seed)() % 2 per step, after
    ``skip`` draws (DominoTiler.cpp:51,70)."""
    return (mt19937_draws(seed, skip + steps)[skip:] % 2).astype(np.uint8)


def mtgp_draws(n_side: int, seed: int, launches: int) -> np.ndarray:
    """The float draws of the 'mtgp' mode for the first ``launches`` half-sweeps of a domino
    walk seeded ``seed`` on an n_side tiling: array (launches, n_side - 2, n_side // 2 - 2),
    entry [h, i-1, m-1] the curand_uniform value candidate site (i, m) receives at
    half-sweep h (dominokernel.cu:14-15)."""
    n = int(n_side)
    out = np.zeros((int(launches), n - 2, n // 2 - 2), np.float32)
    _check(lib().rt_domino_mtgp_draws(n, int(seed), int(launches), _ptr(out)))
    return out


def lozenge_mtgp_draws(n_side: int, seed: int, launches: int) -> np.ndarray:
    """The float draws of the 'mtgp' mode for the first ``launches`` steps of a lozenge walk
    seeded ``seed`` on an n_side tiling: array (launches, n_side, n_side // 3), entry [h, i, j]
    the curand_uniform value slot (i, j) of the rotated colour receives at step h
    (lozengekernel.cu:20-21)."""
    n = int(n_side)
    out = np.zeros((int(launches), n, n // 3), np.float32)
    _check(lib().rt_lozenge_mtgp_draws(n, int(seed), int(launches), _ptr(out)))
    return out


def recttri_mtgp_draws(n_side: int, seed: int, launches: int) -> np.ndarray:
    """The 'mtgp' mode's float draws of a rectangle-triangle walk, laid out as
    lozenge_mtgp_draws (recttrianglekernel.cu:39-40)."""
    n = int(n_side)
    out = np.zeros((int(launches), n, n // 3), np.float32)
    _check(lib().rt_recttri_mtgp_draws(n, int(seed), int(launches), _ptr(out)))
    return out


def td_mtgp_draws(n_side: int, seed: int, launches: int) -> np.ndarray:
    """The 'mtgp' mode's float draws of a bibone walk: array (launches, M, M), M = n_side // 2,
    entry [h, a, b] the curand_uniform value site (a, b) receives at step h."""
    m = int(n_side) // 2
    out = np.zeros((int(launches), m, m), np.float32)
    _check(lib().rt_td_mtgp_draws(int(n_side), int(seed), int(launches), _ptr(out)))
    return out


def SaveMatrix(a, path, rows: int | None = None, cols: int | None = None) -> None:
    """The reference's SaveMatrix (src/common/common.cpp:84-128): without rows/cols the
    square overload (floor(sqrt(size))^2 values)."""
    aa = _i32(a)
    if rows is None:
        _check(lib().rt_save_matrix_square(_ptr(aa), aa.size, str(path).encode()))
    else:
        _check(lib().rt_save_matrix(_ptr(aa), int(rows), int(cols), str(path).encode()))


def LoadMatrix(path) -> np.ndarray:
    """The reference's LoadMatrix (src/common/common.cpp:155-178): every run of digits."""
    n = C.c_int64()
    _check(lib().rt_load_matrix(str(path).encode(), None, 0, C.byref(n)))
    out = np.zeros(n.value, np.int32)
    _check(lib().rt_load_matrix(str(path).encode(), _ptr(out), out.size, C.byref(n)))
    return out


def edge_indicators(t, counts=None) -> np.ndarray:
    """Adds a domino tiling's edge-placement indicators to counts (2 x N x N uint32, created
    when None): [0] horizontal dominoes by the vertex above their middle edge, [1] vertical
    dominoes by the vertex left of their middle edge."""
    tt = _i32(t)
    n = side_of(tt)
    if counts is None:
        counts = np.zeros(2 * n * n, np.uint32)
    _check(lib().rt_domino_edge_indicators(_ptr(tt), n, _ptr(counts)))
    return counts


def aztec_edge_probs(order: int, a: float = 1.0, b: float = 1.0) -> np.ndarray:
    """Exact edge-placement probabilities of DominoTiler.AztecDiamond(order) under the weights
    a / b of the two-periodic rule (a = b: uniform), in the layout of edge_indicators, so that
    counts / samples estimates them (rt_domino_aztec_edge_probs: generalized domino shuffling
    on the device)."""
    n = 2 * int(order) + 6
    out = np.zeros(2 * n * n, np.float64)
    _check(lib().rt_domino_aztec_edge_probs(int(order), float(a), float(b), _ptr(out), out.size, None))
    return out


def tune_load(path) -> None:
    """Loads the autotuner's table of launch shapes (rt_tune_load)."""
    _check(lib().rt_tune_load(str(path).encode()))


def tune_clear() -> None:
    _check(lib().rt_tune_clear())


def tune_lookup(n_side: int, chains: int, rng: str = "tinymt", model: int = 0) -> dict | None:
    """The table's {engine, bands, threads} for a domino sampler of that side, or None."""
    out = np.zeros(3, np.int32)
    if lib().rt_tune_lookup(int(model), int(n_side), int(chains), RNG_MODES[rng], _ptr(out)) != RT_OK:
        return None
    return {"engine": int(out[0]), "bands": int(out[1]), "threads": int(out[2])}


def mt19937_draws(seed: int, count: int) -> np.ndarray:
    """First ``count`` outputs of std::mt19937(seed) (numpy's legacy MT19937 uses the same
    integer seeding and returns raw 32-bit outputs for the full uint32 range)."""
    rs = np.random.RandomState(seed & 0xFFFFFFFF)
    return rs.randint(0, 2**32, size=count, dtype=np.uint32)


__all__ = ["DominoTiler", "DominoSampler", "LozengeTiler", "RectTriangleTiler", "SixVertexTiler", "TriangleDimerTiler", "cftp_batch", "Server", "RTError", "lib", "read_tinymt_params", "mt19937_colours",
           "mt19937_draws", "mtgp_draws", "tune_load", "tune_clear", "tune_lookup", "lozenge_mtgp_draws", "recttri_mtgp_draws",
           "td_mtgp_draws", "CftpStats"]
