"""ctypes binding of the CPU oracle (oracle/polybench_oracle.c).

TEST INFRASTRUCTURE ONLY: imported by tests/, __graft_entry__.smoke() and
bench.py's CPU-baseline leg, never by the product path.
"""
from __future__ import annotations

import ctypes as ct
import subprocess
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
LIB = HERE / "_build" / "liboracle.so"

_f32p = np.ctypeslib.ndpointer(np.float32, flags="C_CONTIGUOUS")
_f64p = np.ctypeslib.ndpointer(np.float64, flags="C_CONTIGUOUS")
_L = ct.c_long

_SIGS = {
    "orc_percent_diff": (ct.c_float, [ct.c_double, ct.c_double]),
    "orc_verify": (_L, [_f32p, _f32p, _L, ct.c_double, ct.POINTER(ct.c_float), ct.POINTER(_L)]),
    "orc_gemm_init": (None, [_f32p, _f32p, _f32p, _L]),
    "orc_mm2_init": (None, [_f32p, _f32p, _f32p, _f32p, _L]),
    "orc_mm3_init": (None, [_f32p, _f32p, _f32p, _f32p, _L]),
    "orc_syrk_init": (None, [_f32p, _f32p, _L]),
    "orc_syr2k_init": (None, [_f32p, _f32p, _f32p, _L]),
    "orc_gemm_host": (None, [_f32p, _f32p, _f32p, _L]),
    "orc_mm2_host": (None, [_f32p, _f32p, _f32p, _f32p, _f32p, _L]),
    "orc_mm3_host": (None, [_f32p, _f32p, _f32p, _f32p, _f32p, _f32p, _f32p, _L]),
    "orc_syrk_host": (None, [_f32p, _f32p, _L]),
    "orc_syr2k_host": (None, [_f32p, _f32p, _f32p, _L]),
    "orc_gemm_body": (None, [_f32p, _f32p, _f32p, _L, _L, _L, ct.c_float, ct.c_float]),
    "orc_syrk_body": (None, [_f32p, _f32p, _L, _L, _L, ct.c_float, ct.c_float]),
    "orc_syr2k_body": (None, [_f32p, _f32p, _f32p, _L, _L, _L, ct.c_float, ct.c_float]),
    "orc_gemm_f64": (None, [ct.c_int, ct.c_int, _L, _L, _L, ct.c_double, _f32p, _L, _f32p, _L, ct.c_void_p,
                            ct.c_void_p, ct.c_double, ct.c_void_p, _L, _f64p, _L]),
    "orc_gemm_f64d": (None, [_L, _L, _L, ct.c_double, _f64p, _L, _f64p, _L, ct.c_double, ct.c_void_p, _L, _f64p,
                             _L]),
    "orc_error_norms": (None, [_f32p, _f64p, _L, ct.POINTER(ct.c_double), ct.POINTER(ct.c_double),
                               ct.POINTER(ct.c_double)]),
    "orc_num_threads": (ct.c_int, []),
    "orc_covariance_init": (None, [_f32p, _L]),
    "orc_covariance_host": (None, [_f32p, _f32p, _f32p, _L]),
    "orc_correlation_init": (None, [_f32p, _L]),
    "orc_correlation_host": (None, [_f32p, _f32p, _f32p, _f32p, _L]),
    "orc_matmulchain_product": (None, [_f32p, _f32p, _f32p, _L]),
    "orc_atax_init": (None, [_f32p, _f32p, _L]),
    "orc_atax_host": (None, [_f32p, _f32p, _f32p, _f32p, _L]),
    "orc_bicg_init": (None, [_f32p, _f32p, _f32p, _L]),
    "orc_bicg_host": (None, [_f32p, _f32p, _f32p, _f32p, _f32p, _L]),
    "orc_mvt_init": (None, [_f32p, _f32p, _f32p, _f32p, _f32p, _L]),
    "orc_mvt_host": (None, [_f32p, _f32p, _f32p, _f32p, _f32p, _L]),
    "orc_gesummv_init": (None, [_f32p, _f32p, _f32p, _L]),
    "orc_gesummv_host": (None, [_f32p, _f32p, _f32p, _f32p, _f32p, _L]),
}

_lib = None


LIB_FAST = HERE / "_build" / "liboracle_fast.so"
_fast = None


def build(target: Path = LIB) -> Path:
    subprocess.run(["make", "-s", "-C", str(HERE), str(target.relative_to(HERE))], check=True)
    return target


def _load(path: Path) -> ct.CDLL:
    if not path.exists() or path.stat().st_mtime < (HERE / "polybench_oracle.c").stat().st_mtime:
        build(path)
    l = ct.CDLL(str(path))
    for name, (res, args) in _SIGS.items():
        f = getattr(l, name)
        f.restype = res
        f.argtypes = args
    return l


def lib() -> ct.CDLL:
    """The strict build (-ffp-contract=off): the oracle proper."""
    global _lib
    if _lib is None:
        _lib = _load(LIB)
    return _lib


def fast_lib() -> ct.CDLL:
    """The reference's release-flag build (-O3 -ffast-math; no -march=native), for timing only."""
    global _fast
    if _fast is None:
        _fast = _load(LIB_FAST)
    return _fast


def f32(shape) -> np.ndarray:
    return np.zeros(shape, dtype=np.float32)


def percent_diff(v1: float, v2: float) -> float:
    return float(lib().orc_percent_diff(v1, v2))


def verify(host: np.ndarray, dev: np.ndarray, threshold: float = 0.05):
    """Reference verify loop: (first failing flat index or -1, max percentDiff, failing count)."""
    md = ct.c_float()
    nf = _L()
    first = lib().orc_verify(np.ascontiguousarray(host, np.float32), np.ascontiguousarray(dev, np.float32),
                             host.size, threshold, ct.byref(md), ct.byref(nf))
    return int(first), float(md.value), int(nf.value)


# ---- per-benchmark initialisers: return the arrays the reference's setup() fills
def init_gemm(n):
    A, B, C = f32((n, n)), f32((n, n)), f32((n, n))
    lib().orc_gemm_init(A, B, C, n)
    return A, B, C


def init_mm2(n):
    A, B, C, D = (f32((n, n)) for _ in range(4))
    lib().orc_mm2_init(A, B, C, D, n)
    return A, B, C, D


def init_mm3(n):
    A, B, C, D = (f32((n, n)) for _ in range(4))
    lib().orc_mm3_init(A, B, C, D, n)
    return A, B, C, D


def init_syrk(n):
    A, C = f32((n, n)), f32((n, n))
    lib().orc_syrk_init(A, C, n)
    return A, C


def init_syr2k(n):
    A, B, C = f32((n, n)), f32((n, n)), f32((n, n))
    lib().orc_syr2k_init(A, B, C, n)
    return A, B, C


# ---- host reference loops (the reference's verify() oracles)
def host_gemm(n):
    A, B, C = init_gemm(n)
    lib().orc_gemm_host(A, B, C, n)
    return C


def host_mm2(n):
    A, B, C, D = init_mm2(n)
    E = f32((n, n))
    lib().orc_mm2_host(A, B, C, D, E, n)
    return E


def host_mm3(n):
    A, B, C, D = init_mm3(n)
    E, F, G = f32((n, n)), f32((n, n)), f32((n, n))
    lib().orc_mm3_host(A, B, C, D, E, F, G, n)
    return G


def host_syrk(n):
    A, C = init_syrk(n)
    lib().orc_syrk_host(A, C, n)
    return C


def host_syr2k(n):
    A, B, C = init_syr2k(n)
    lib().orc_syr2k_host(A, B, C, n)
    return C


# ---- FP64 references
def init_covariance(n):
    """The (n+1) x (n+1) data array covariance.cpp's setup() fills."""
    data = f32((n + 1, n + 1))
    lib().orc_covariance_init(data, n)
    return data


def host_covariance(n, data=None):
    """covariance.cpp's host loop on its own init (or on `data`): the (n+1) x (n+1) symmat."""
    data = init_covariance(n) if data is None else np.array(data, np.float32, copy=True)
    symmat, mean = f32((n + 1, n + 1)), f32(n + 1)
    lib().orc_covariance_host(data, symmat, mean, n)
    return symmat


def init_correlation(n):
    """The (n+1) x (n+1) data array correlation.cpp's setup() fills (row stride n)."""
    data = f32((n + 1, n + 1))
    lib().orc_correlation_init(data, n)
    return data


def host_correlation(n, data=None):
    """correlation.cpp's host loop on its own init (or on `data`): the (n+1) x (n+1) symmat."""
    data = init_correlation(n) if data is None else np.array(data, np.float32, copy=True)
    mean, stddev, symmat = f32(n + 1), f32(n + 1), f32((n + 1, n + 1))
    lib().orc_correlation_host(data, mean, stddev, symmat, n)
    return symmat


def matmulchain_product(a, b):
    """matmulchain.cpp's multiply kernel (int accumulator) on n x n float matrices."""
    n = a.shape[0]
    c = f32((n, n))
    lib().orc_matmulchain_product(np.ascontiguousarray(a, np.float32), np.ascontiguousarray(b, np.float32), c, n)
    return c


# ---- matrix-vector benchmarks: init returns the setup() arrays, host the verify-loop outputs
def init_atax(n):
    x, A = f32(n), f32((n, n))
    lib().orc_atax_init(x, A, n)
    return A, x


def host_atax(n):
    A, x = init_atax(n)
    y, tmp = f32(n), f32(n)
    lib().orc_atax_host(A, x, y, tmp, n)
    return y


def init_bicg(n):
    A, p, r = f32((n, n)), f32(n), f32(n)
    lib().orc_bicg_init(A, p, r, n)
    return A, p, r


def host_bicg(n):
    """s then q, concatenated."""
    A, p, r = init_bicg(n)
    s, q = f32(n), f32(n)
    lib().orc_bicg_host(A, r, s, p, q, n)
    return np.concatenate([s, q])


def init_mvt(n):
    a, x1, x2, y1, y2 = f32((n, n)), f32(n), f32(n), f32(n), f32(n)
    lib().orc_mvt_init(a, x1, x2, y1, y2, n)
    return a, x1, x2, y1, y2


def host_mvt(n):
    """x1 then x2, concatenated."""
    a, x1, x2, y1, y2 = init_mvt(n)
    lib().orc_mvt_host(a, x1, x2, y1, y2, n)
    return np.concatenate([x1, x2])


def init_gesummv(n):
    A, B, x = f32((n, n)), f32((n, n)), f32(n)
    lib().orc_gesummv_init(A, B, x, n)
    return A, B, x


def host_gesummv(n):
    A, B, x = init_gesummv(n)
    y, tmp = f32(n), f32(n)
    lib().orc_gesummv_host(A, B, x, y, tmp, n)
    return y


def gemm_f64(A, B, C0=None, alpha=1.0, beta=0.0, op_a=0, op_b=0, A2=None, B2=None):
    """alpha * op(A) op(B) [+ op(A2) op(B2)] + beta * C0 in float64 (FP32 inputs)."""
    A = np.ascontiguousarray(A, np.float32)
    B = np.ascontiguousarray(B, np.float32)
    M = A.shape[1] if op_a else A.shape[0]
    K = A.shape[0] if op_a else A.shape[1]
    N = B.shape[0] if op_b else B.shape[1]
    out = np.empty((M, N), np.float64)
    c0 = np.ascontiguousarray(C0, np.float32) if C0 is not None else None
    a2 = np.ascontiguousarray(A2, np.float32) if A2 is not None else None
    b2 = np.ascontiguousarray(B2, np.float32) if B2 is not None else None
    lib().orc_gemm_f64(op_a, op_b, M, N, K, alpha, A, A.shape[1], B, B.shape[1],
                       a2.ctypes.data if a2 is not None else None, b2.ctypes.data if b2 is not None else None,
                       beta, c0.ctypes.data if c0 is not None else None, N, out, N)
    return out


def gemm_f64d(A, B, C0=None, alpha=1.0, beta=0.0):
    A = np.ascontiguousarray(A, np.float64)
    B = np.ascontiguousarray(B, np.float64)
    M, K = A.shape
    N = B.shape[1]
    out = np.empty((M, N), np.float64)
    c0 = np.ascontiguousarray(C0, np.float64) if C0 is not None else None
    lib().orc_gemm_f64d(M, N, K, alpha, A, K, B, N, beta, c0.ctypes.data if c0 is not None else None, N, out, N)
    return out


def error_norms(C, R):
    """(max|C-R|/max|R|, ||C-R||_F/||R||_F, max elementwise |C-R|/|R|)."""
    a, b, c = ct.c_double(), ct.c_double(), ct.c_double()
    lib().orc_error_norms(np.ascontiguousarray(C, np.float32), np.ascontiguousarray(R, np.float64), C.size,
                          ct.byref(a), ct.byref(b), ct.byref(c))
    return float(a.value), float(b.value), float(c.value)


def num_threads() -> int:
    return int(lib().orc_num_threads())
