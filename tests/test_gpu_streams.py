"""GPU random streams against the oracle: PCG32 words and Sobol integers bit-exact,
normals to the precision of each transform."""
import ctypes as C

import numpy as np
import pytest

from oracle import loader

pytestmark = pytest.mark.gpu


def _gpu_words(native, seed, stream, first, count):
    out = np.zeros(count, np.uint32)
    native.check(native.lib.kgpu_pcg_words(native.handle, seed, stream, first, count,
                                           out.ctypes.data_as(C.POINTER(C.c_uint32))))
    return out


def _gpu_normals(native, seed, block, first, count, precision):
    out = np.zeros(count, np.float64)
    native.check(native.lib.kgpu_pcg_normals(native.handle, seed, block, first, count, precision,
                                             out.ctypes.data_as(C.POINTER(C.c_double))))
    return out


@pytest.mark.parametrize("seed,stream,first", [(42, 0, 0), (1009, 255, 12345),
                                               (2**64 - 1, 4095, 2**40 + 3), (7, 2**40, 999)])
def test_pcg_words_bit_exact(native, seed, stream, first):
    assert np.array_equal(_gpu_words(native, seed, stream, first, 4096),
                          loader.pcg_words(seed, stream, first, 4096))


@pytest.mark.parametrize("block,first", [(0, 0), (3, 1), (4095, 252 * 255 + 1)])
def test_pcg_normals(native, block, first):
    ref = loader.pcg_normals(1729, block, first, 2048)
    fp64 = _gpu_normals(native, 1729, block, first, 2048, 0)
    fp32 = _gpu_normals(native, 1729, block, first, 2048, 1)
    # FP64: identical words and polynomial; CUDA log vs glibc log differ by <= 1 ulp.
    assert np.max(np.abs(fp64 - ref)) < 1e-14
    # FP32: hardware log/sin/cos on the same words.
    assert np.max(np.abs(fp32 - ref)) < 2e-5


@pytest.mark.parametrize("dims,dim,first", [(504, 0, 0), (504, 503, 1 << 19), (21201, 21200, 7)])
def test_sobol_points(native, dims, dim, first):
    count = 4096
    bits = np.zeros(count, np.uint64)
    n64 = np.zeros(count, np.float64)
    n32 = np.zeros(count, np.float64)
    P = C.POINTER
    native.check(native.lib.kgpu_sobol_points(native.handle, 42, dims, dim, first, count,
                                              bits.ctypes.data_as(P(C.c_uint64)),
                                              n64.ctypes.data_as(P(C.c_double)), 0))
    native.check(native.lib.kgpu_sobol_points(native.handle, 42, dims, dim, first, count, None,
                                              n32.ctypes.data_as(P(C.c_double)), 1))
    rbits, rnorm = loader.sobol_points(42, dims, dim, first, count)
    assert np.array_equal(bits, rbits)
    assert np.max(np.abs(n64 - rnorm)) < 1e-13
    assert np.max(np.abs(n32 - rnorm) / np.maximum(1.0, np.abs(rnorm))) < 2e-5
