"""Seeded synthetic inputs for the structural-scan workloads (libpars_synth.so).

The generators are host C++ (pars_gb300/csrc/synth.cpp); every function here is a
pure function of its seed and parameters, identical on x86 and Arm.

Workload families (sizes are parameters; the defaults below are the named
workloads used by bench.py and the tests):

* ``json_doc``  — JSON tree, 40% objects / 30% arrays / 30% scalars, fanout
  U[1,8], depth <= 16, keys 4-12 lowercase bytes, strings 0-64 bytes of which 5%
  carry escaped quotes / backslash runs of 1-4, ints and floats, 0-2 spaces or
  newlines between tokens, wrapped in one top-level array (64 MiB single document).
* ``json_deep`` — depth drawn up to 1024 per top-level spine, ~20% of bytes in
  1-64 KiB strings with escape runs (2 GiB stress document).
* ``csv_doc``   — 16 columns, LF records, unquoted fields U[0,24] alphanumerics,
  10% quoted fields with ',', LF and '""' at 5% per position (1 GiB).
* ``config_doc`` — TOML / C-like / INI / XML documents for the general-path
  grammars (64 MiB each in bench.py).
* ``json_batch`` — many json_doc-style documents with log-normal sizes (median
  2 KiB, sigma 1.5, clamped 64 B - 4 MiB), concatenated with a uint64 offset table.
"""
from __future__ import annotations

import ctypes
import os

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
_LIB = None


def _lib():
    global _LIB
    if _LIB is None:
        path = os.path.join(_HERE, "libpars_synth.so")
        if not os.path.exists(path):
            raise ImportError(
                f"{path} is missing: run `python -c 'import __graft_entry__ as g; g.build()'`")
        L = ctypes.CDLL(path)
        u64, vp = ctypes.c_uint64, ctypes.c_void_p
        L.pars_synth_json.restype = u64
        L.pars_synth_json.argtypes = [u64, u64, ctypes.c_int, vp, u64]
        L.pars_synth_csv.restype = u64
        L.pars_synth_csv.argtypes = [u64, u64, vp, u64]
        L.pars_synth_config.restype = u64
        L.pars_synth_config.argtypes = [u64, ctypes.c_int, u64, vp, u64]
        L.pars_synth_alpha.restype = None
        L.pars_synth_alpha.argtypes = [u64, vp, u64, vp, u64]
        L.pars_synth_lognormal_sizes.restype = None
        L.pars_synth_lognormal_sizes.argtypes = [u64, u64, ctypes.c_double, ctypes.c_double,
                                                 u64, u64, vp]
        _LIB = L
    return _LIB


def _gen(fn, *args, target: int, slack: int) -> np.ndarray:
    cap = target + slack
    while True:
        buf = np.empty(cap, np.uint8)
        n = fn(*args, buf.ctypes.data, cap)
        if n <= cap:
            return buf[:n]
        cap = int(n) + 64


def json_doc(seed: int, target: int) -> np.ndarray:
    return _gen(lambda s, t, p, c: _lib().pars_synth_json(s, t, 0, p, c), seed, target,
                target=target, slack=64 * 1024 + target // 64)


def json_deep(seed: int, target: int) -> np.ndarray:
    return _gen(lambda s, t, p, c: _lib().pars_synth_json(s, t, 1, p, c), seed, target,
                target=target, slack=2 * 1024 * 1024 + target // 64)


def csv_doc(seed: int, target: int) -> np.ndarray:
    return _gen(lambda s, t, p, c: _lib().pars_synth_csv(s, t, p, c), seed, target,
                target=target, slack=8192)


_CONFIG_KINDS = {"toml": 0, "clike": 1, "ini": 2, "xml": 3}


def config_doc(grammar: str, seed: int, target: int) -> np.ndarray:
    """A document for one of the multi-descriptor grammars (toml, clike, ini, xml):
    every lexical mode (strings, literal strings, comments, tags) with the grammar's
    structural bytes both inside and outside them."""
    kind = _CONFIG_KINDS[grammar]
    return _gen(lambda s, t, p, c: _lib().pars_synth_config(s, kind, t, p, c), seed, target,
                target=target, slack=4096)


def alpha(seed: int, alphabet: bytes, n: int) -> np.ndarray:
    a = np.frombuffer(alphabet, np.uint8).copy()
    out = np.empty(n, np.uint8)
    if n:
        _lib().pars_synth_alpha(seed, a.ctypes.data, a.size, out.ctypes.data, n)
    return out


def lognormal_sizes(seed: int, count: int, median: float = 2048.0, sigma: float = 1.5,
                    lo: int = 64, hi: int = 4 << 20) -> np.ndarray:
    out = np.empty(count, np.uint64)
    _lib().pars_synth_lognormal_sizes(seed, count, median, sigma, lo, hi, out.ctypes.data)
    return out


def json_batch(seed: int, count: int, median: float = 2048.0, sigma: float = 1.5):
    """Concatenated json_doc-style documents; returns (bytes, uint64 offsets[count+1])."""
    sizes = lognormal_sizes(seed, count, median, sigma)
    parts = []
    offs = np.zeros(count + 1, np.uint64)
    total = 0
    for i, sz in enumerate(sizes.tolist()):
        d = json_doc(seed * 1000003 + i + 1, int(sz))
        parts.append(d)
        total += d.size
        offs[i + 1] = total
    return (np.concatenate(parts) if parts else np.zeros(0, np.uint8)), offs
