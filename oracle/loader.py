"""TEST INFRASTRUCTURE: ctypes loader of the FP64 CPU oracle (liboracle.so).

Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg import this module.
"""
import ctypes as C
import os
import subprocess
import threading

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
_LIB = None
_LOCK = threading.Lock()


def build() -> str:
    """Compiles liboracle.so with the committed Makefile (seconds)."""
    subprocess.run(["make", "-s", "-C", HERE], check=True)
    return os.path.join(HERE, "liboracle.so")


def load():
    global _LIB
    with _LOCK:
        if _LIB is not None:
            return _LIB
        path = os.path.join(HERE, "liboracle.so")
        sources = [os.path.join(HERE, f) for f in ("oracle.cpp", "lsmc.cpp", "oracle_core.h",
                                                  "heston_adi.cpp", "mlp.cpp", "Makefile")]
        sources.append(os.path.join(HERE, "..", "include", "kgpu.h"))
        newest = max(os.path.getmtime(s) for s in sources if os.path.exists(s))
        if not os.path.exists(path) or os.path.getmtime(path) < newest:
            build()
        from kiyosi_gb300 import abi
        lib = C.CDLL(path)
        P = C.POINTER
        lib.kor_price_book.argtypes = [P(abi.Model), P(abi.Book), P(abi.Settings),
                                       P(abi.Estimate), C.c_int]
        lib.kor_price_book.restype = C.c_int
        lib.kor_pcg_words.argtypes = [C.c_uint64, C.c_uint64, C.c_uint64, C.c_int64,
                                      P(C.c_uint32)]
        lib.kor_pcg_normals.argtypes = [C.c_uint64, C.c_uint64, C.c_uint64, C.c_int64,
                                        P(C.c_double)]
        lib.kor_sobol_points.argtypes = [C.c_uint64, C.c_int, C.c_int, C.c_uint64, C.c_int64,
                                         P(C.c_uint64), P(C.c_double)]
        lib.kor_sin_cos_turns.argtypes = [C.c_double, P(C.c_double), P(C.c_double)]
        lib.kor_ndtri.argtypes = [C.c_double]
        lib.kor_ndtri.restype = C.c_double
        lib.kor_golden_european_v019.argtypes = [C.c_uint64, C.c_int64] + [C.c_double] * 6 + [
            C.c_int, C.c_int]
        lib.kor_golden_european_v019.restype = C.c_double
        if hasattr(lib, "kor_lsmc_price"):
            lib.kor_lsmc_price.argtypes = [P(abi.Model), C.c_double, C.c_double, C.c_double,
                                           P(abi.LsmcSettings), C.c_uint64, P(abi.LsmcResult),
                                           C.c_int]
            lib.kor_lsmc_price.restype = C.c_int
        if hasattr(lib, "kor_heston_adi_american"):
            lib.kor_heston_adi_american.argtypes = [P(abi.Model), C.c_double, C.c_double,
                                                    C.c_double, C.c_int, C.c_int, C.c_int,
                                                    C.c_int]
            lib.kor_heston_adi_american.restype = C.c_double
        lib.kor_price_shared_group.argtypes = [P(abi.Model), P(abi.Book), P(abi.Settings),
                                               C.c_double, C.c_double, P(C.c_int32),
                                               P(C.c_int32), P(C.c_int32), P(C.c_double),
                                               C.c_int, P(C.c_double), P(C.c_double), C.c_int]
        lib.kor_price_shared_group.restype = C.c_int
        lib.kor_mlp_gradients.argtypes = [P(C.c_float), P(C.c_float), C.c_int, C.c_int,
                                          P(C.c_double)]
        lib.kor_mlp_gradients.restype = C.c_double
        _LIB = lib
        return lib


def price_book(ctx, packed, settings, threads=0):
    """Prices a PackedBook on the CPU oracle; returns a list of abi.Estimate."""
    from kiyosi_gb300 import abi
    lib = load()
    n = len(packed.contracts)
    out = (abi.Estimate * n)()
    model = ctx.kgpu_model()
    book = packed.struct()
    status = lib.kor_price_book(C.byref(model), C.byref(book), C.byref(settings), out, threads)
    if status != 0:
        from kiyosi_gb300.errors import raise_for_status
        raise_for_status(status, "oracle")
    return list(out)


def price_shared_group(ctx, packed, settings, strips=None, threads=0):
    """One shared daily grid's lanes (the contracts of `packed`) walked by the oracle's
    restatement of the multi-lane path loop.  `strips` gives per lane None or
    (kind, ascending log levels) with kind 1 = knock-out, 2 = knock-in.  Returns the lane
    prices and, per lane, the strip members' prices (or None)."""
    from kiyosi_gb300 import abi
    from kiyosi_gb300.market import safe_log_returns
    lib = load()
    n = len(packed.contracts)
    strips = strips or [None] * n
    kind = np.zeros(n, np.int32)
    offset = np.zeros(n, np.int32)
    length = np.zeros(n, np.int32)
    levels = []
    for i, strip in enumerate(strips):
        if strip is not None:
            kind[i], offset[i], length[i] = strip[0], len(levels), len(strip[1])
            levels.extend(strip[1])
    levels = np.array(levels + [0.0], np.float64)
    lane_prices = np.zeros(n, np.float64)
    strip_prices = np.zeros(len(levels), np.float64)
    low, high = safe_log_returns(ctx.spot)
    model = ctx.kgpu_model()
    book = packed.struct()
    I32, F64 = C.POINTER(C.c_int32), C.POINTER(C.c_double)
    status = lib.kor_price_shared_group(C.byref(model), C.byref(book), C.byref(settings), low, high,
                                        kind.ctypes.data_as(I32), offset.ctypes.data_as(I32),
                                        length.ctypes.data_as(I32), levels.ctypes.data_as(F64),
                                        len(levels) - 1, lane_prices.ctypes.data_as(F64),
                                        strip_prices.ctypes.data_as(F64), threads)
    if status != 0:
        from kiyosi_gb300.errors import raise_for_status
        raise_for_status(status, "oracle")
    members = [None if strip is None else list(strip_prices[offset[i]:offset[i] + length[i]])
               for i, strip in enumerate(strips)]
    return list(lane_prices), members


def pcg_normals(seed, block, first, count):
    lib = load()
    out = np.zeros(count, np.float64)
    lib.kor_pcg_normals(seed, block, first, count, out.ctypes.data_as(C.POINTER(C.c_double)))
    return out


def pcg_words(seed, stream, first, count):
    lib = load()
    out = np.zeros(count, np.uint32)
    lib.kor_pcg_words(seed, stream, first, count, out.ctypes.data_as(C.POINTER(C.c_uint32)))
    return out


def sobol_points(seed, dims, dim, first, count):
    lib = load()
    bits = np.zeros(count, np.uint64)
    normals = np.zeros(count, np.float64)
    lib.kor_sobol_points(seed, dims, dim, first, count,
                         bits.ctypes.data_as(C.POINTER(C.c_uint64)),
                         normals.ctypes.data_as(C.POINTER(C.c_double)))
    return bits, normals


def mlp_gradients(params, samples, bf16_operands=True):
    """Loss and gradients of the LSMC continuation network on a batch (float32 inputs:
    params[4481], samples[n][4] = (x0, x1, x2, target))."""
    lib = load()
    params = np.ascontiguousarray(params, np.float32)
    samples = np.ascontiguousarray(samples, np.float32)
    grads = np.zeros(params.size, np.float64)
    loss = lib.kor_mlp_gradients(params.ctypes.data_as(C.POINTER(C.c_float)),
                                 samples.ctypes.data_as(C.POINTER(C.c_float)), len(samples),
                                 int(bf16_operands), grads.ctypes.data_as(C.POINTER(C.c_double)))
    return loss, grads


def mlp_adam(params, samples, batch, steps, learning_rate, beta1=0.9, beta2=0.999, eps=1e-8):
    """`steps` Adam steps (Kingma and Ba, zero initial moments) on the LSMC continuation
    network, minibatch b being samples [b * batch, ...) cycled in order, with the
    gradients of mlp_gradients (the tensor-core kernel's BF16 operand rounding) and the
    moments, bias corrections and update in float32 as the training kernel keeps them.
    Returns the parameters after the last step."""
    p = np.array(params, np.float32)
    x = np.ascontiguousarray(samples, np.float32)
    m = np.zeros_like(p)
    v = np.zeros_like(p)
    per_epoch = (len(x) + batch - 1) // batch
    b1, b2, e, lr = np.float32(beta1), np.float32(beta2), np.float32(eps), np.float32(learning_rate)
    one = np.float32(1.0)
    for step in range(steps):
        first = (step % per_epoch) * batch
        _, g = mlp_gradients(p, x[first:first + batch])
        g = g.astype(np.float32)
        m = b1 * m + (one - b1) * g
        v = b2 * v + (one - b2) * g * g
        t = np.float32(step + 1)
        bias1 = one - np.float32(b1 ** t)
        bias2 = one - np.float32(b2 ** t)
        p = (p - lr * (m / bias1) / (np.sqrt(v / bias2) + e)).astype(np.float32)
    return p
