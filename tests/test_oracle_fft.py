"""Known-answer tests for the oracle FFT (oracle/offt.c), which restates the
unscaled complex DFT of the reference's absent fft_3d/FFTW 2.1.5 dependency
(poisson.cpp:87,431,453).  Pinned against numpy.fft."""
import ctypes

import numpy as np
import pytest


@pytest.fixture(scope="module")
def offt(oracle_lib):
    L = oracle_lib.lib()
    L.offt_3d.argtypes = [ctypes.POINTER(ctypes.c_double), ctypes.c_int, ctypes.c_int,
                          ctypes.c_int, ctypes.c_int]

    def fft3(a, sign):
        buf = np.ascontiguousarray(np.stack([a.real, a.imag], axis=-1), dtype=np.float64)
        nz, ny, nx = a.shape
        L.offt_3d(buf.ctypes.data_as(ctypes.POINTER(ctypes.c_double)), nx, ny, nz, sign)
        return buf[..., 0] + 1j * buf[..., 1]

    return fft3


@pytest.mark.parametrize("shape", [(8, 8, 8), (12, 16, 24), (5, 6, 30), (16, 48, 10),
                                   (1, 1, 96), (2, 3, 128)])
def test_matches_numpy(offt, shape):
    rng = np.random.default_rng(1)
    a = rng.standard_normal(shape) + 1j * rng.standard_normal(shape)
    ref = np.fft.fftn(a)
    got = offt(a, -1)
    assert np.abs(got - ref).max() <= 1e-13 * np.abs(ref).max()
    back = offt(ref, +1)
    assert np.abs(back - a * a.size).max() <= 1e-13 * a.size * np.abs(a).max()


def test_single_mode_and_parseval(offt):
    nz, ny, nx = 12, 10, 16
    k = np.arange(nx)[None, None, :]
    j = np.arange(ny)[None, :, None]
    z = np.arange(nz)[:, None, None]
    a = np.exp(2j * np.pi * (3 * k / nx + 2 * j / ny + 5 * z / nz)) * np.ones((nz, ny, nx))
    A = offt(a, -1)
    peak = np.zeros((nz, ny, nx), complex)
    peak[5, 2, 3] = a.size
    assert np.abs(A - peak).max() < 1e-11
    rng = np.random.default_rng(2)
    r = rng.standard_normal((nz, ny, nx))
    R = offt(r.astype(complex), -1)
    assert abs((np.abs(R) ** 2).sum() / r.size - (r ** 2).sum()) < 1e-10 * (r ** 2).sum()
