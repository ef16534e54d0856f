"""The library after cudaDeviceReset.

An application may tear its device context down with cudaDeviceReset and go
on.  What the library set up once per device (kernels' shared-memory
opt-ins, the number of resident CTA pairs, the device address of the
allocation-free entry point's array) belongs to the old context; it is
remembered with the context's id and redone in the new one.  In a fresh
process: the plain FP32 kernel, a CTA-pair bf16x3 launch and the
allocation-free entry point give the same bits after the reset as before.
"""
import subprocess
import sys
from pathlib import Path

import pytest

pytestmark = pytest.mark.gpu

PKG = Path(__file__).resolve().parent.parent / "sycl-bench_gb300"

SCRIPT = r'''
import ctypes as ct, sys
import numpy as np
sys.path.insert(0, sys.argv[1])
import gbpoly
from gbpoly import Op, Precision

rt = ct.CDLL("libcudart.so.13")
rng = np.random.default_rng(5)
cases = [  # (form, M, N, K): the SIMT kernel; CTA pairs (80 pair tiles, K = 512: configuration 3)
    (Precision.FP32, 512, 640, 384), (Precision.BF16X3, 2048, 2560, 512)]
data = {c: tuple(rng.standard_normal(s).astype(np.float32) for s in ((c[1], c[3]), (c[3], c[2]), (c[1], c[2])))
        for c in cases}

def run():
    out = []
    with gbpoly.Context(0) as ctx:
        for (prec, M, N, K), (A, B, C) in data.items():
            dA, dB, dC = ctx.upload(A), ctx.upload(B), ctx.upload(C)
            ctx.gemm(prec, M, N, K, 1.5, dA, K, dB, N, 0.5, dC, N)
            ctx.synchronize()
            out.append(ctx.download(dC, (M, N)))
        (_, M, N, K), (A, B, C) = list(data.items())[0]
        dA, dB, dC = ctx.upload(A), ctx.upload(B), ctx.upload(C)
        st = ctx.lib.gbpoly_gemm_f32_bf16x3_noalloc(ctx.handle, 0, 0, M, N, K, ct.c_float(1.5), ct.c_void_p(int(dA)), K,
                                                    ct.c_void_p(int(dB)), N, ct.c_float(0.5), ct.c_void_p(int(dC)), N)
        assert st == 0, ctx.lib.gbpoly_last_error()
        ctx.synchronize()
        out.append(ctx.download(dC, (M, N)))
    return out

before = run()
assert rt.cudaDeviceReset() == 0
after = run()
for x, y in zip(before, after):
    assert np.array_equal(x, y)
print("same after reset")
'''


def test_same_results_after_device_reset():
    r = subprocess.run([sys.executable, "-c", SCRIPT, str(PKG)], capture_output=True, text=True, timeout=600)
    assert r.returncode == 0 and "same after reset" in r.stdout, (r.stdout[-2000:], r.stderr[-3000:])
