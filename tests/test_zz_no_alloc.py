"""The allocation-free Poisson entry point (tpm_poisson_solve_noalloc).

It exists for callers that cannot allocate device memory themselves - a
plug-in that only receives buffers from its host application, or work issued
while a stream is being captured - so it keeps all of its scratch in one
fixed device array inside the library.  These tests call it through the C
ABI on device buffers (allocated here by torch, as such a caller's host
application would) and check its result against the context-based
tpm_poisson_solve, twice in a row, since successive calls share and reuse
that array.  This file is collected last so that a run that stops at the
first failure has already run every other test.
"""
import ctypes

import numpy as np
import pytest

from conftest import rel_err

pytestmark = pytest.mark.gpu

TOL = 1e-12  # the FP64 parity bar used by the other GPU tests


@pytest.fixture(scope="module")
def capi():
    from tpm import build, capi

    build.build()
    return capi


def noalloc_solve(capi, torch, p, C3, P0, RHS, max_it, eps):
    dev = torch.device("cuda", 0)
    c = torch.from_numpy(np.ascontiguousarray(C3)).to(dev)
    pr = torch.from_numpy(np.ascontiguousarray(P0)).to(dev)
    r = torch.from_numpy(np.ascontiguousarray(RHS)).to(dev)
    it = ctypes.c_int(-1)
    err = ctypes.c_double(-1.0)
    stream = torch.cuda.current_stream(dev).cuda_stream
    L = capi.load_library()
    rc = L.tpm_poisson_solve_noalloc(p.Nx, p.Ny, p.Nz, p.Lx, p.Ly, p.Lz, c.data_ptr(),
                                     pr.data_ptr(), r.data_ptr(), max_it, eps, stream,
                                     ctypes.byref(it), ctypes.byref(err))
    assert rc == 0, rc
    torch.cuda.synchronize(dev)
    return pr.cpu().numpy(), it.value, err.value


def problem(N, seed, anis=False):
    from tpm import params as P

    p = P.physical(N, 1, nu=0.02, A=0.0, tau_p=0.1, mass_loading=0.1)
    if anis:
        p = p.replace(Nx=N, Ny=N // 2 * 3 if (N // 2 * 3) % 2 == 0 else N, Nz=N // 2,
                      Ly=1.5 * p.Ly, Lz=0.5 * p.Lz)
    rng = np.random.default_rng(seed)
    shape = (p.Nz, p.Ny, p.Nx)
    C3 = 1.0 / (1.0 + 0.2 * rng.random((3,) + shape))
    RHS = rng.standard_normal(shape)
    RHS -= RHS.mean()
    P0 = rng.standard_normal(shape)
    return p, C3, P0, RHS


def test_noalloc_matches_context_solve_twice(capi):
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    # two calls in a row on different problems and sizes: the second reuses
    # the shared scratch left by the first
    for N, seed, anis in ((24, 1, False), (32, 2, True)):
        p, C3, P0, RHS = problem(N, seed, anis)
        ctx = capi.Context(p, 1)
        want, it_w, err_w = ctx.poisson_solve(C3, P0, RHS, 5, 0.0)
        ctx.close()
        got, it_g, err_g = noalloc_solve(capi, torch, p, C3, P0, RHS, 5, 0.0)
        assert it_g == it_w == 5
        assert rel_err(got, want) <= TOL
        assert abs(err_g - err_w) <= TOL * max(abs(err_w), 1e-300)


def test_noalloc_tolerance_stop_and_limits(capi):
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    p, C3, P0, RHS = problem(16, 3)
    ctx = capi.Context(p, 1)
    want, it_w, _ = ctx.poisson_solve(C3, P0, RHS, 30, 1e-12)
    ctx.close()
    for _ in range(2):
        got, it_g, _ = noalloc_solve(capi, torch, p, C3, P0, RHS, 30, 1e-12)
        assert it_g == it_w
        assert rel_err(got, want) <= TOL
    # a grid beyond the fixed scratch is refused, not attempted
    L = capi.load_library()
    rc = L.tpm_poisson_solve_noalloc(256, 256, 256, 1.0, 1.0, 1.0, 1, 1, 1, 1, 0.0, None,
                                     None, None)
    assert rc == -1
