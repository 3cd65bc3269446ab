"""The allocation-free Poisson entry point (tpm_poisson_solve_noalloc).

It exists for callers that cannot allocate device memory themselves - a
plug-in that only receives buffers from its host application, or a runtime
whose memory pool owns the device - so it keeps all of its scratch in one
fixed device array inside the library.  These tests call it through the C
ABI on device buffers (allocated here by torch, as such a caller's host
application would) and check its result against the context-based
tpm_poisson_solve, twice in a row, since successive calls share and reuse
that array; on a right-hand side with a non-zero mean (used as given, like
the reference's poisson::Solve); on a freshly created stream with work
queued ahead of the call; and that a stream being captured into a CUDA graph
is refused (the call synchronises its stream).  This file is collected last
so that a run that stops at the first failure has already run every other
test.
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


def noalloc_solve(capi, torch, p, C3, P0, RHS, max_it, eps, stream=None):
    dev = torch.device("cuda", 0)
    s = stream if stream is not None else torch.cuda.current_stream(dev)
    with torch.cuda.stream(s):
        c = torch.from_numpy(np.ascontiguousarray(C3)).to(dev)
        pr = torch.from_numpy(np.ascontiguousarray(P0)).to(dev)
        r = torch.from_numpy(np.ascontiguousarray(RHS)).to(dev)
    it = ctypes.c_int(-1)
    err = ctypes.c_double(-1.0)
    stream = s.cuda_stream
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


def test_noalloc_nonzero_mean_rhs_on_a_fresh_stream(capi):
    """A right-hand side with a non-zero mean, on a newly created stream that
    has a long copy queued ahead of the call (the solve must wait for it, as
    stream order says), twice in a row; and iteration counts and the error
    reported as the context solve reports them."""
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    dev = torch.device("cuda", 0)
    p, C3, P0, RHS = problem(30, 4)
    RHS = RHS + 0.37  # mean kept: poisson::Solve uses RHS as given
    ctx = capi.Context(p, 1)
    want, it_w, err_w = ctx.poisson_solve(C3, P0, RHS, 4, 0.0)
    ctx.close()
    s = torch.cuda.Stream(dev)
    big = torch.empty(1 << 27, dtype=torch.float32, device=dev)
    for _ in range(2):
        with torch.cuda.stream(s):
            big.fill_(1.0)  # work queued on the stream ahead of the solve
            big.mul_(2.0)
        got, it_g, err_g = noalloc_solve(capi, torch, p, C3, P0, RHS, 4, 0.0, stream=s)
        assert it_g == it_w == 4
        assert rel_err(got, want) <= TOL
        assert abs(err_g - err_w) <= TOL * max(abs(err_w), 1e-300)
    assert float(big[-1]) == 2.0
    # no iteration: P unchanged, the reference's initial error 100 reported
    got, it_g, err_g = noalloc_solve(capi, torch, p, C3, P0, RHS, 0, 0.0, stream=s)
    assert it_g == 0 and err_g == 100.0
    assert np.array_equal(got, P0)


def test_noalloc_refuses_a_capturing_stream(capi):
    """The call synchronises its stream, which a stream capture forbids: on a
    capturing stream it returns TPM_ERR_STATE without issuing any work, and
    the capture stays valid."""
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    dev = torch.device("cuda", 0)
    p, C3, P0, RHS = problem(16, 5)
    c = torch.from_numpy(C3).to(dev)
    pr = torch.from_numpy(P0).to(dev)
    r = torch.from_numpy(RHS).to(dev)
    x = torch.zeros(16, device=dev)
    L = capi.load_library()
    s = torch.cuda.Stream(dev)
    g = torch.cuda.CUDAGraph()
    rcs = []
    with torch.cuda.stream(s):
        torch.cuda.synchronize(dev)
        with torch.cuda.graph(g, stream=s):
            x.add_(1.0)
            rcs.append(L.tpm_poisson_solve_noalloc(p.Nx, p.Ny, p.Nz, p.Lx, p.Ly, p.Lz,
                                                   c.data_ptr(), pr.data_ptr(), r.data_ptr(),
                                                   3, 0.0, s.cuda_stream, None, None))
    assert rcs == [-6]  # TPM_ERR_STATE
    g.replay()
    torch.cuda.synchronize(dev)
    assert float(x[0]) == 1.0
    assert np.array_equal(pr.cpu().numpy(), P0)
