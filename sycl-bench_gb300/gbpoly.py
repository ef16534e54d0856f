"""ctypes binding of libgbpoly (the C ABI in include/gbpoly.h).

This is the Python face of the same boundary the C++ PolyBench executables
use.  It loads the in-tree ``lib/libgbpoly.so`` and fails loudly if that
library has not been built: there is no fallback implementation.

    from gbpoly import Context, Precision
    with Context(0) as ctx:
        A = ctx.upload(a_np); B = ctx.upload(b_np); C = ctx.upload(c_np)
        ctx.gemm(Precision.FP32, M, N, K, 32412.0, A, K, B, N, 2123.0, C, N)
        out = ctx.download(C, (M, N))
"""
from __future__ import annotations

import ctypes as ct
import enum
import os
from pathlib import Path

import numpy as np

PKG = Path(__file__).resolve().parent
LIB_PATH = PKG / "lib" / "libgbpoly.so"


class GbpolyError(RuntimeError):
    def __init__(self, status: int, message: str):
        super().__init__(f"gbpoly status {status}: {message}")
        self.status = status


class Status(enum.IntEnum):
    OK = 0
    INVALID = 1
    CUDA = 2
    NOMEM = 3
    TIMEOUT = 4
    UNSUPPORTED = 5
    STATE = 6


class Precision(enum.IntEnum):
    FP32 = 0
    BF16X3 = 1
    TF32 = 2
    FP8 = 3
    TF32X3 = 4
    BF16X6 = 5
    FP16X3 = 6


class Op(enum.IntEnum):
    N = 0
    T = 1


_c_i64 = ct.c_int64
_vp = ct.c_void_p


class GemmDesc(ct.Structure):
    """gbpoly_gemm_desc: C = alpha * op(A) op(B) + beta * C."""
    _fields_ = [("op_a", ct.c_int), ("op_b", ct.c_int), ("M", ct.c_int64), ("N", ct.c_int64), ("K", ct.c_int64),
                ("alpha", ct.c_float), ("beta", ct.c_float), ("A", ct.c_void_p), ("lda", ct.c_int64),
                ("B", ct.c_void_p), ("ldb", ct.c_int64), ("C", ct.c_void_p), ("ldc", ct.c_int64)]

class GemvTerm(ct.Structure):
    """gbpoly_gemv_term: y = beta * y + alpha * op(A) x."""
    _fields_ = [("op", ct.c_int), ("alpha", ct.c_float), ("beta", ct.c_float), ("x", ct.c_void_p),
                ("y", ct.c_void_p)]


# name -> (restype, argtypes); every exported symbol of include/gbpoly.h
SIGNATURES: dict[str, tuple] = {
    "gbpoly_init": (ct.c_int, [ct.c_int, ct.POINTER(_vp)]),
    "gbpoly_destroy": (ct.c_int, [_vp]),
    "gbpoly_last_error": (ct.c_char_p, []),
    "gbpoly_device_name": (ct.c_int, [_vp, ct.c_char_p, ct.c_size_t]),
    "gbpoly_device_props": (ct.c_int, [_vp] + [ct.POINTER(ct.c_int)] * 4),
    "gbpoly_synchronize": (ct.c_int, [_vp]),
    "gbpoly_set_stream": (ct.c_int, [_vp, _vp]),
    "gbpoly_malloc": (ct.c_int, [_vp, ct.POINTER(_vp), ct.c_size_t]),
    "gbpoly_free": (ct.c_int, [_vp, _vp]),
    "gbpoly_host_alloc": (ct.c_int, [_vp, ct.POINTER(_vp), ct.c_size_t]),
    "gbpoly_host_free": (ct.c_int, [_vp, _vp]),
    "gbpoly_memcpy_h2d": (ct.c_int, [_vp, _vp, _vp, ct.c_size_t]),
    "gbpoly_memcpy_d2h": (ct.c_int, [_vp, _vp, _vp, ct.c_size_t]),
    "gbpoly_memcpy_d2d": (ct.c_int, [_vp, _vp, _vp, ct.c_size_t]),
    "gbpoly_memset": (ct.c_int, [_vp, _vp, ct.c_int, ct.c_size_t]),
    "gbpoly_workspace_reserve": (ct.c_int, [_vp, ct.c_size_t]),
    "gbpoly_workspace_query": (ct.c_int, [ct.c_int, _c_i64, _c_i64, _c_i64, ct.c_int, ct.POINTER(ct.c_size_t)]),
    "gbpoly_gemm_config_count": (ct.c_int, [ct.c_int, ct.POINTER(ct.c_int)]),
    "gbpoly_gemm_config_set": (ct.c_int, [_vp, ct.c_int, _c_i64, _c_i64, _c_i64, ct.c_int]),
    "gbpoly_gemm_config_get": (ct.c_int, [_vp, ct.c_int, _c_i64, _c_i64, _c_i64, ct.POINTER(ct.c_int)]),
    "gbpoly_autotune_gemm": (ct.c_int, [_vp, ct.c_int, _c_i64, _c_i64, _c_i64, ct.c_int, ct.POINTER(ct.c_int),
                                        ct.POINTER(ct.c_float)]),
    "gbpoly_autotune_save": (ct.c_int, [_vp, ct.c_char_p]),
    "gbpoly_autotune_load": (ct.c_int, [_vp, ct.c_char_p, ct.POINTER(ct.c_int)]),
    "gbpoly_graph_begin": (ct.c_int, [_vp]),
    "gbpoly_graph_end": (ct.c_int, [_vp, ct.POINTER(_vp)]),
    "gbpoly_graph_launch": (ct.c_int, [_vp, _vp]),
    "gbpoly_graph_destroy": (ct.c_int, [_vp, _vp]),
    "gbpoly_event_create": (ct.c_int, [_vp, ct.POINTER(_vp)]),
    "gbpoly_event_destroy": (ct.c_int, [_vp, _vp]),
    "gbpoly_event_record": (ct.c_int, [_vp, _vp]),
    "gbpoly_event_elapsed_ms": (ct.c_int, [_vp, _vp, _vp, ct.POINTER(ct.c_float)]),
    "gbpoly_profile_enable": (ct.c_int, [_vp, ct.c_int]),
    "gbpoly_tail_split_enable": (ct.c_int, [_vp, ct.c_int]),
    "gbpoly_profile_read": (ct.c_int, [_vp, ct.c_int, ct.c_char_p, ct.POINTER(ct.c_int), ct.POINTER(ct.c_double),
                                       ct.POINTER(ct.c_int)]),
    "gbpoly_gemm_f32": (ct.c_int, [_vp, ct.c_int, ct.c_int, ct.c_int, _c_i64, _c_i64, _c_i64, ct.c_float, _vp,
                                   _c_i64, _vp, _c_i64, ct.c_float, _vp, _c_i64]),
    "gbpoly_gemm_f32_host": (ct.c_int, [_vp, ct.c_int, ct.c_int, ct.c_int, _c_i64, _c_i64, _c_i64, ct.c_float, _vp,
                                        _c_i64, _vp, _c_i64, ct.c_float, _vp, _c_i64]),
    "gbpoly_syrk_f32": (ct.c_int, [_vp, ct.c_int, _c_i64, _c_i64, ct.c_float, _vp, _c_i64, ct.c_float, _vp,
                                   _c_i64]),
    "gbpoly_syr2k_f32": (ct.c_int, [_vp, ct.c_int, _c_i64, _c_i64, ct.c_float, _vp, _c_i64, _vp, _c_i64,
                                    ct.c_float, _vp, _c_i64]),
    "gbpoly_stream_hold": (ct.c_int, [_vp, ct.c_uint32]),
    "gbpoly_stream_release": (ct.c_int, [_vp]),
    "gbpoly_wait_probe": (ct.c_int, [_vp, ct.c_uint32]),
    "gbpoly_gemv_f32": (ct.c_int, [_vp, ct.c_int, _c_i64, _c_i64, ct.c_float, _vp, _c_i64, _vp, ct.c_float, _vp]),
    "gbpoly_atax_f32": (ct.c_int, [_vp, _c_i64, _c_i64, _vp, _c_i64, _vp, _vp, _vp]),
    "gbpoly_gemv_pair_f32": (ct.c_int, [_vp, _c_i64, _c_i64, _vp, _c_i64, _vp, ct.c_int]),
    "gbpoly_gesummv_f32": (ct.c_int, [_vp, _c_i64, _c_i64, ct.c_float, _vp, _c_i64, _vp, _c_i64, _vp, ct.c_float, _vp,
                                      _vp]),
    "gbpoly_column_mean_f32": (ct.c_int, [_vp, _c_i64, _c_i64, _vp, _c_i64, ct.c_float, _vp]),
    "gbpoly_column_stddev_f32": (ct.c_int, [_vp, _c_i64, _c_i64, _vp, _c_i64, _vp, ct.c_float, ct.c_float, _vp]),
    "gbpoly_center_columns_f32": (ct.c_int, [_vp, _c_i64, _c_i64, _vp, _c_i64, _vp, _vp, ct.c_float, _vp, _c_i64]),
    "gbpoly_set_diagonal_f32": (ct.c_int, [_vp, _c_i64, ct.c_float, _vp, _c_i64]),
    "gbpoly_covariance_f32": (ct.c_int, [_vp, ct.c_int, _c_i64, _c_i64, _vp, _c_i64, _vp, _vp, ct.c_float, _vp,
                                         _c_i64]),
    "gbpoly_grouped_plan": (ct.c_int, [_vp, ct.c_int, _vp, ct.c_int, ct.POINTER(_vp)]),
    "gbpoly_grouped_run": (ct.c_int, [_vp, _vp]),
    "gbpoly_grouped_info": (ct.c_int, [_vp, ct.POINTER(ct.c_int64), ct.POINTER(ct.c_int), ct.POINTER(ct.c_size_t)]),
    "gbpoly_grouped_destroy": (ct.c_int, [_vp, _vp]),
    "gbpoly_gemm_grouped_f32": (ct.c_int, [_vp, ct.c_int, _vp, ct.c_int]),
    "gbpoly_grouped_config_of": (ct.c_int, [_vp, ct.POINTER(ct.c_int)]),
    "gbpoly_grouped_config_count": (ct.c_int, [ct.c_int, ct.POINTER(ct.c_int)]),
    "gbpoly_grouped_config_set": (ct.c_int, [_vp, ct.c_int, _vp, ct.c_int, ct.c_int]),
    "gbpoly_grouped_config_get": (ct.c_int, [_vp, ct.c_int, _vp, ct.c_int, ct.POINTER(ct.c_int)]),
    "gbpoly_autotune_grouped": (ct.c_int, [_vp, ct.c_int, _vp, ct.c_int, ct.c_int, ct.POINTER(ct.c_int),
                                           ct.POINTER(ct.c_float)]),
    "gbpoly_gemm_f32_bf16x3_noalloc": (ct.c_int, [_vp, ct.c_int, ct.c_int, _c_i64, _c_i64, _c_i64, ct.c_float, _vp,
                                                  _c_i64, _vp, _c_i64, ct.c_float, _vp, _c_i64]),
    "gbpoly_gemm_f64": (ct.c_int, [_vp, ct.c_int, ct.c_int, _c_i64, _c_i64, _c_i64, ct.c_double, _vp, _c_i64, _vp,
                                   _c_i64, ct.c_double, _vp, _c_i64]),
    "gbpoly_syrk_f64": (ct.c_int, [_vp, _c_i64, _c_i64, ct.c_double, _vp, _c_i64, ct.c_double, _vp, _c_i64]),
    "gbpoly_syr2k_f64": (ct.c_int, [_vp, _c_i64, _c_i64, ct.c_double, _vp, _c_i64, _vp, _c_i64, ct.c_double, _vp,
                                    _c_i64]),
    "gbpoly_convert_f32_f64": (ct.c_int, [_vp, _vp, _vp, _c_i64]),
    "gbpoly_error_norms": (ct.c_int, [_vp, _vp, _c_i64, _vp, _c_i64, _c_i64, _c_i64, ct.POINTER(ct.c_double),
                                      ct.POINTER(ct.c_double), ct.POINTER(ct.c_double)]),
}

_lib = None


def load_library(path: Path | None = None) -> ct.CDLL:
    """Load libgbpoly.so and bind every signature; raise if it is missing."""
    global _lib
    if _lib is not None and path is None:
        return _lib
    p = Path(path or os.environ.get("GBPOLY_LIB", LIB_PATH))
    if not p.exists():
        raise RuntimeError(f"libgbpoly.so not found at {p}: build it with "
                           f"`python -c 'import __graft_entry__ as g; g.build()'`")
    lib = ct.CDLL(str(p))
    for name, (res, args) in SIGNATURES.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    if path is None:
        _lib = lib
    return lib


def _check(status: int) -> None:
    if status != 0:
        msg = _lib.gbpoly_last_error().decode(errors="replace") if _lib else ""
        raise GbpolyError(status, msg)


class DeviceBuffer:
    """Owning handle of a device allocation made through gbpoly_malloc."""

    def __init__(self, ctx: "Context", nbytes: int):
        self.ctx = ctx
        self.nbytes = nbytes
        p = _vp()
        _check(ctx.lib.gbpoly_malloc(ctx.handle, ct.byref(p), nbytes))
        self.ptr = p.value or 0

    def free(self) -> None:
        if self.ptr:
            _check(self.ctx.lib.gbpoly_free(self.ctx.handle, _vp(self.ptr)))
            self.ptr = 0

    def __int__(self) -> int:
        return self.ptr


class Event:
    def __init__(self, ctx: "Context"):
        self.ctx = ctx
        h = _vp()
        _check(ctx.lib.gbpoly_event_create(ctx.handle, ct.byref(h)))
        self.handle = h

    def record(self) -> None:
        _check(self.ctx.lib.gbpoly_event_record(self.ctx.handle, self.handle))

    def elapsed_ms(self, end: "Event") -> float:
        ms = ct.c_float()
        _check(self.ctx.lib.gbpoly_event_elapsed_ms(self.ctx.handle, self.handle, end.handle, ct.byref(ms)))
        return float(ms.value)

    def destroy(self) -> None:
        if self.handle:
            self.ctx.lib.gbpoly_event_destroy(self.ctx.handle, self.handle)
            self.handle = None


def _ptr(x) -> _vp:
    if isinstance(x, DeviceBuffer):
        return _vp(x.ptr)
    if isinstance(x, np.ndarray):
        return _vp(x.ctypes.data)
    return _vp(int(x) if x else None)


class Context:
    """One device, one stream.  Mirrors the reference's BenchmarkArgs::device_queue."""

    def __init__(self, device: int = 0):
        self.lib = load_library()
        h = _vp()
        _check(self.lib.gbpoly_init(device, ct.byref(h)))
        self.handle = h
        self._buffers: list[DeviceBuffer] = []

    # -- lifetime
    def close(self) -> None:
        if self.handle:
            for b in self._buffers:
                try:
                    b.free()
                except GbpolyError:
                    pass
            self._buffers.clear()
            self.lib.gbpoly_destroy(self.handle)
            self.handle = None

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    # -- device info
    def device_name(self) -> str:
        buf = ct.create_string_buffer(256)
        _check(self.lib.gbpoly_device_name(self.handle, buf, 256))
        return buf.value.decode()

    def device_props(self) -> dict:
        v = [ct.c_int() for _ in range(4)]
        _check(self.lib.gbpoly_device_props(self.handle, *[ct.byref(x) for x in v]))
        return {"sm_count": v[0].value, "sm_clock_khz": v[1].value, "cc": (v[2].value, v[3].value)}

    def synchronize(self) -> None:
        _check(self.lib.gbpoly_synchronize(self.handle))

    # -- memory
    def alloc(self, nbytes: int) -> DeviceBuffer:
        b = DeviceBuffer(self, nbytes)
        self._buffers.append(b)
        return b

    def free(self, buf: DeviceBuffer) -> None:
        buf.free()
        if buf in self._buffers:
            self._buffers.remove(buf)

    def upload(self, arr: np.ndarray) -> DeviceBuffer:
        arr = np.ascontiguousarray(arr)
        b = self.alloc(arr.nbytes)
        self.h2d(b, arr)
        self.synchronize()
        return b

    def h2d(self, dst, src: np.ndarray, nbytes: int | None = None) -> None:
        _check(self.lib.gbpoly_memcpy_h2d(self.handle, _ptr(dst), _ptr(src), src.nbytes if nbytes is None else nbytes))

    def d2h(self, dst: np.ndarray, src, nbytes: int | None = None) -> None:
        _check(self.lib.gbpoly_memcpy_d2h(self.handle, _ptr(dst), _ptr(src), dst.nbytes if nbytes is None else nbytes))

    def download(self, buf, shape, dtype=np.float32) -> np.ndarray:
        out = np.empty(shape, dtype=dtype)
        self.d2h(out, buf)
        self.synchronize()
        return out

    def memset(self, buf, value: int, nbytes: int) -> None:
        _check(self.lib.gbpoly_memset(self.handle, _ptr(buf), value, nbytes))

    def profile(self, enable: bool) -> None:
        _check(self.lib.gbpoly_profile_enable(self.handle, 1 if enable else 0))

    def profile_read(self) -> dict[str, tuple[int, float]]:
        """{kernel: (launches, total ms)} since the last read."""
        cap = 32
        names = ct.create_string_buffer(64 * cap)
        counts = (ct.c_int * cap)()
        tot = (ct.c_double * cap)()
        n = ct.c_int()
        _check(self.lib.gbpoly_profile_read(self.handle, cap, names, counts, tot, ct.byref(n)))
        out = {}
        for i in range(min(n.value, cap)):
            nm = names.raw[64 * i:64 * i + 64].split(b"\0", 1)[0].decode()
            out[nm] = (counts[i], tot[i])
        return out

    def workspace_reserve(self, nbytes: int) -> None:
        _check(self.lib.gbpoly_workspace_reserve(self.handle, nbytes))

    def workspace_query(self, prec, M, N, K, same_operand=False) -> int:
        v = ct.c_size_t()
        _check(self.lib.gbpoly_workspace_query(int(prec), M, N, K, 1 if same_operand else 0, ct.byref(v)))
        return int(v.value)

    def config_count(self, prec) -> int:
        v = ct.c_int()
        _check(self.lib.gbpoly_gemm_config_count(int(prec), ct.byref(v)))
        return v.value

    def tail_split(self, enable: bool) -> None:
        """K-split units for the last round of CTA-pair tiles (default on)."""
        _check(self.lib.gbpoly_tail_split_enable(self.handle, 1 if enable else 0))

    def config_set(self, prec, M, N, K, config: int) -> None:
        _check(self.lib.gbpoly_gemm_config_set(self.handle, int(prec), M, N, K, config))

    def config_get(self, prec, M, N, K) -> int:
        v = ct.c_int()
        _check(self.lib.gbpoly_gemm_config_get(self.handle, int(prec), M, N, K, ct.byref(v)))
        return v.value

    def autotune(self, prec, M, N, K, reps: int = 3) -> tuple[int, float]:
        c, ms = ct.c_int(), ct.c_float()
        _check(self.lib.gbpoly_autotune_gemm(self.handle, int(prec), M, N, K, reps, ct.byref(c), ct.byref(ms)))
        return c.value, ms.value

    def autotune_save(self, path) -> None:
        _check(self.lib.gbpoly_autotune_save(self.handle, str(path).encode()))

    def autotune_load(self, path) -> int:
        n = ct.c_int()
        _check(self.lib.gbpoly_autotune_load(self.handle, str(path).encode(), ct.byref(n)))
        return n.value

    # -- grouped contractions
    @staticmethod
    def descs(items) -> ct.Array:
        """items: dicts with M, N, K, alpha, beta, A, lda, B, ldb, C, ldc[, op_a, op_b] (device buffers or ints)."""
        arr = (GemmDesc * len(items))()
        for d, it in zip(arr, items):
            d.op_a, d.op_b = int(it.get("op_a", Op.N)), int(it.get("op_b", Op.N))
            d.M, d.N, d.K = it["M"], it["N"], it["K"]
            d.alpha, d.beta = it["alpha"], it["beta"]
            d.A, d.lda = int(it["A"]) or None, it["lda"]
            d.B, d.ldb = int(it["B"]) or None, it["ldb"]
            d.C, d.ldc = int(it["C"]) or None, it["ldc"]
        return arr

    def grouped_plan(self, prec, descs):
        h = _vp()
        _check(self.lib.gbpoly_grouped_plan(self.handle, int(prec), ct.cast(descs, _vp), len(descs), ct.byref(h)))
        return h

    def grouped_run(self, plan) -> None:
        _check(self.lib.gbpoly_grouped_run(self.handle, plan))

    def grouped_info(self, plan) -> dict:
        f, t, b = ct.c_int64(), ct.c_int(), ct.c_size_t()
        _check(self.lib.gbpoly_grouped_info(plan, ct.byref(f), ct.byref(t), ct.byref(b)))
        return {"flops": f.value, "tiles": t.value, "device_bytes": b.value}

    def grouped_config_of(self, plan) -> int:
        c = ct.c_int()
        _check(self.lib.gbpoly_grouped_config_of(plan, ct.byref(c)))
        return c.value

    def grouped_config_count(self, prec) -> int:
        c = ct.c_int()
        _check(self.lib.gbpoly_grouped_config_count(int(prec), ct.byref(c)))
        return c.value

    def grouped_config_set(self, prec, descs, config: int) -> None:
        _check(self.lib.gbpoly_grouped_config_set(self.handle, int(prec), ct.cast(descs, _vp), len(descs), config))

    def grouped_config_get(self, prec, descs) -> int:
        c = ct.c_int()
        _check(self.lib.gbpoly_grouped_config_get(self.handle, int(prec), ct.cast(descs, _vp), len(descs),
                                                  ct.byref(c)))
        return c.value

    def autotune_grouped(self, prec, descs, reps: int = 3) -> tuple[int, float]:
        """Time every grouped tile configuration on these problems (C is overwritten); keep the fastest."""
        c, ms = ct.c_int(), ct.c_float()
        _check(self.lib.gbpoly_autotune_grouped(self.handle, int(prec), ct.cast(descs, _vp), len(descs), reps,
                                                ct.byref(c), ct.byref(ms)))
        return c.value, ms.value

    def grouped_destroy(self, plan) -> None:
        _check(self.lib.gbpoly_grouped_destroy(self.handle, plan))

    def graph_begin(self) -> None:
        _check(self.lib.gbpoly_graph_begin(self.handle))

    def graph_end(self):
        g = _vp()
        _check(self.lib.gbpoly_graph_end(self.handle, ct.byref(g)))
        return g

    def graph_launch(self, g) -> None:
        _check(self.lib.gbpoly_graph_launch(self.handle, g))

    def graph_destroy(self, g) -> None:
        _check(self.lib.gbpoly_graph_destroy(self.handle, g))

    def event(self) -> Event:
        return Event(self)

    # -- contractions (asynchronous; call synchronize() to wait and to collect errors)
    def gemm(self, prec, M, N, K, alpha, A, lda, B, ldb, beta, C, ldc, op_a=Op.N, op_b=Op.N) -> None:
        _check(self.lib.gbpoly_gemm_f32(self.handle, int(prec), int(op_a), int(op_b), M, N, K, alpha, _ptr(A), lda,
                                        _ptr(B), ldb, beta, _ptr(C), ldc))

    def gemm_host(self, prec, M, N, K, alpha, A, lda, B, ldb, beta, C, ldc, op_a=Op.N, op_b=Op.N) -> None:
        """A, B, C are host pointers (numpy arrays or ints)."""
        _check(self.lib.gbpoly_gemm_f32_host(self.handle, int(prec), int(op_a), int(op_b), M, N, K, alpha, _ptr(A), lda,
                                             _ptr(B), ldb, beta, _ptr(C), ldc))

    def syrk(self, prec, N, K, alpha, A, lda, beta, C, ldc) -> None:
        _check(self.lib.gbpoly_syrk_f32(self.handle, int(prec), N, K, alpha, _ptr(A), lda, beta, _ptr(C), ldc))

    def syr2k(self, prec, N, K, alpha, A, lda, B, ldb, beta, C, ldc) -> None:
        _check(self.lib.gbpoly_syr2k_f32(self.handle, int(prec), N, K, alpha, _ptr(A), lda, _ptr(B), ldb, beta,
                                         _ptr(C), ldc))

    # -- stream hold (device-only timing of a group of launches)
    def stream_hold(self, timeout_us: int = 20000) -> None:
        _check(self.lib.gbpoly_stream_hold(self.handle, timeout_us))

    def stream_release(self) -> None:
        _check(self.lib.gbpoly_stream_release(self.handle))

    def wait_probe(self, limit_us: int) -> None:
        """Queue a bounded wait that runs out after limit_us (the next synchronize reports TIMEOUT)."""
        _check(self.lib.gbpoly_wait_probe(self.handle, limit_us))

    # -- matrix-vector products (atax, bicg, mvt, gesummv)
    def gemv(self, op, rows, cols, alpha, A, lda, x, beta, y) -> None:
        _check(self.lib.gbpoly_gemv_f32(self.handle, int(op), rows, cols, alpha, _ptr(A), lda, _ptr(x), beta, _ptr(y)))

    def atax(self, rows, cols, A, lda, x, tmp, y) -> None:
        _check(self.lib.gbpoly_atax_f32(self.handle, rows, cols, _ptr(A), lda, _ptr(x), _ptr(tmp), _ptr(y)))

    def gemv_pair(self, rows, cols, A, lda, terms) -> None:
        """terms: up to two (op, alpha, beta, x, y) tuples, all over one pass of A."""
        arr = (GemvTerm * len(terms))()
        for t, (op, alpha, beta, x, y) in zip(arr, terms):
            t.op, t.alpha, t.beta, t.x, t.y = int(op), alpha, beta, _ptr(x).value, _ptr(y).value
        _check(self.lib.gbpoly_gemv_pair_f32(self.handle, rows, cols, _ptr(A), lda, ct.cast(arr, _vp), len(terms)))

    def gesummv(self, rows, cols, alpha, A, lda, B, ldb, x, beta, tmp, y) -> None:
        _check(self.lib.gbpoly_gesummv_f32(self.handle, rows, cols, alpha, _ptr(A), lda, _ptr(B), ldb, _ptr(x), beta,
                                           _ptr(tmp), _ptr(y)))

    # -- column statistics (covariance / correlation passes)
    def column_mean(self, rows, cols, X, ldx, divisor, mean) -> None:
        _check(self.lib.gbpoly_column_mean_f32(self.handle, rows, cols, _ptr(X), ldx, divisor, _ptr(mean)))

    def column_stddev(self, rows, cols, X, ldx, mean, divisor, eps, stddev) -> None:
        _check(self.lib.gbpoly_column_stddev_f32(self.handle, rows, cols, _ptr(X), ldx, _ptr(mean), divisor, eps,
                                                 _ptr(stddev)))

    def covariance(self, prec, rows, cols, X, ldx, mean, stddev, scale_div, C, ldc) -> None:
        """C = Y^T Y, Y the centred (stddev None) or centred and scaled columns of X."""
        _check(self.lib.gbpoly_covariance_f32(self.handle, int(prec), rows, cols, _ptr(X), ldx, _ptr(mean),
                                              _ptr(stddev) if stddev is not None else None, scale_div, _ptr(C), ldc))

    def center_columns(self, rows, cols, X, ldx, mean, stddev, scale_div, Y, ldy) -> None:
        _check(self.lib.gbpoly_center_columns_f32(self.handle, rows, cols, _ptr(X), ldx, _ptr(mean),
                                                  _ptr(stddev) if stddev is not None else None, scale_div, _ptr(Y),
                                                  ldy))

    def set_diagonal(self, n, value, C, ldc) -> None:
        _check(self.lib.gbpoly_set_diagonal_f32(self.handle, n, value, _ptr(C), ldc))

    # -- FP64
    def gemm_f64(self, M, N, K, alpha, A, lda, B, ldb, beta, C, ldc, op_a=Op.N, op_b=Op.N) -> None:
        _check(self.lib.gbpoly_gemm_f64(self.handle, int(op_a), int(op_b), M, N, K, alpha, _ptr(A), lda, _ptr(B), ldb,
                                        beta, _ptr(C), ldc))

    def syrk_f64(self, N, K, alpha, A, lda, beta, C, ldc) -> None:
        _check(self.lib.gbpoly_syrk_f64(self.handle, N, K, alpha, _ptr(A), lda, beta, _ptr(C), ldc))

    def syr2k_f64(self, N, K, alpha, A, lda, B, ldb, beta, C, ldc) -> None:
        _check(self.lib.gbpoly_syr2k_f64(self.handle, N, K, alpha, _ptr(A), lda, _ptr(B), ldb, beta, _ptr(C), ldc))

    def convert_f32_f64(self, src, dst, count: int) -> None:
        _check(self.lib.gbpoly_convert_f32_f64(self.handle, _ptr(src), _ptr(dst), count))

    def error_norms(self, C, ldc, R, ldr, rows, cols) -> tuple[float, float, float]:
        a, b, c = ct.c_double(), ct.c_double(), ct.c_double()
        _check(self.lib.gbpoly_error_norms(self.handle, _ptr(C), ldc, _ptr(R), ldr, rows, cols, ct.byref(a),
                                           ct.byref(b), ct.byref(c)))
        return float(a.value), float(b.value), float(c.value)
