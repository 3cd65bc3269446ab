"""Whole-step CUDA graphs, the FFT tile autotuner and batched ensembles.

Every one of these changes only how the kernels are launched, never what they
compute, so the bar is bit-identical fields, particles and scalars against
eager stepping of the same boxes.
"""
import numpy as np
import pytest

from golden import load
from tpm import inputs, params as P

pytestmark = pytest.mark.gpu

FIELDS = ("RU", "RU_INT", "RHO", "P", "C", "Q")


@pytest.fixture(scope="module")
def capi():
    from tpm import build, capi

    build.build()
    return capi


def case(dims=(32, 32, 32), npart=5000, seed=3, heat=0.5, eps=1e-13, prec=P.PREC_FP64, **extra):
    nx, ny, nz = dims
    p = P.physical(nx, npart, nu=0.02, A=0.1, tau_p=0.1, mass_loading=0.5, heating_Q=heat,
                   iterations=20, epsilon=eps, precision=prec)
    if (ny, nz) != (nx, nx):
        p = p.replace(Ny=ny, Nz=nz, Ly=p.Lx * ny / nx, Lz=p.Lx * nz / nx)
    s = inputs.make_state(p, npart, seed=seed)
    return p.replace(dt=inputs.cfl_dt(p, s.RU), **extra), s


def state(ctx):
    out = {f: ctx.download_field(f) for f in FIELDS}
    out.update({"p_" + k: v for k, v in ctx.download_particles("base").items()})
    sc = ctx.scalars()
    out.update({k: sc[k] for k in ("P0", "T_cur", "num_timestep", "last_poisson_iterations",
                                   "total_poisson_iterations")})
    return out


def assert_same(a, b):
    assert a.keys() == b.keys()
    for k in a:
        assert np.array_equal(np.asarray(a[k]), np.asarray(b[k])), k


def run(capi, p, s, nsteps, graph=False, autotune=False):
    ctx = capi.Context(p, s.npart)
    ctx.load(s)
    if autotune:
        ctx.autotune()
    ctx.initialize()
    if graph:
        ctx.set_graph(True)
    ctx.run(nsteps)
    ctx.sync()
    return ctx


@pytest.mark.parametrize("prec,eps", [(P.PREC_FP64, 1e-13), (P.PREC_FP64, 0.0),
                                      (P.PREC_MIXED, 1e-13)])
def test_graph_steps_bit_identical_to_eager(capi, prec, eps):
    p, s = case(prec=prec, eps=eps)
    eager = run(capi, p, s, 5)
    graph = run(capi, p, s, 5, graph=True)
    assert_same(state(graph), state(eager))
    # the Poisson loop is a conditional while node: its body is enqueued once
    # per solve and repeats on the device, so fewer launches are issued
    assert graph.launch_count() <= eager.launch_count()
    if eps > 0:
        assert 0 < graph.scalars()["last_poisson_iterations"] < 20


def test_graph_follows_the_parameter_switch(capi):
    # threshold crossed after the first step: A, g and Iteration change (params.cpp:80-86)
    p, s, _, _, _ = load("cooled24_gravity_switch")
    eager = run(capi, p, s, 4)
    graph = run(capi, p, s, 4, graph=True)
    assert_same(state(graph), state(eager))


def test_graph_then_eager_then_graph(capi):
    p, s = case(dims=(24, 30, 16), npart=3000, seed=4)
    eager = run(capi, p, s, 6)
    ctx = capi.Context(p, s.npart)
    ctx.load(s)
    ctx.initialize()
    ctx.set_graph(True)
    ctx.run(2)
    ctx.set_graph(False)
    ctx.run(1)
    ctx.set_graph(True)
    ctx.run(3)
    ctx.sync()
    assert_same(state(ctx), state(eager))


def test_autotune_keeps_results(capi):
    p, s = case(dims=(64, 64, 64), npart=20_000, seed=5)
    ref = run(capi, p, s, 2)
    tuned = run(capi, p, s, 2, autotune=True)
    assert_same(state(tuned), state(ref))
    pens = tuned.autotune()
    assert len(pens) == 6 and all(1 <= q <= 32 for q in pens[:3])
    assert all(t in (128, 256, 512) for t in pens[3:])


@pytest.mark.parametrize("dims", [(32, 48, 40), (32, 32, 256)])
def test_fft_tma_tiles_keep_results(capi, dims):
    """The mixed path's y and z passes with TMA tiles (the default; at 256
    points the z pass with its middle stages in registers) and with plain
    tiles give the same bits, eagerly and from graphs, and after autotuning."""
    p, s = case(prec=P.PREC_MIXED, dims=dims, npart=4000, seed=8)
    ref = state(run(capi, p, s, 3))
    for graph in (False, True):
        ctx = capi.Context(p, s.npart)
        ctx.load(s)
        ctx.set_option(capi.OPT_FFT_TMA, 0)
        ctx.initialize()
        if graph:
            ctx.set_graph(True)
        ctx.run(3)
        ctx.sync()
        assert_same(state(ctx), ref)
    assert_same(state(run(capi, p, s, 3, graph=True, autotune=True)), ref)


@pytest.mark.parametrize("prec", [P.PREC_FP64, P.PREC_MIXED])
def test_fixed_fft_tiles_keep_results(capi, prec):
    # pencils 1, 2, 4 and odd thread counts against the default tiles
    p, s = case(prec=prec, dims=(32, 48, 40), npart=4000, seed=6)
    ref = run(capi, p, s, 3)
    for tiles in ([1, 2, 4, 64, 96, 160], [4, 1, 2, 256, 32, 512]):
        ctx = capi.Context(p, s.npart)
        ctx.load(s)
        ctx.set_fft_tiles(tiles)
        ctx.initialize()
        ctx.run(3)
        ctx.sync()
        assert_same(state(ctx), state(ref))
    ctx = capi.Context(p, s.npart)
    for bad in ([3, 1, 1, 128, 128, 128], [1, 1, 1, 100, 128, 128], [1, 1, 1, 128, 2048, 128],
                [0, 1, 1, 128, 128, 128], [1, 1, 4096, 128, 128, 128]):
        with pytest.raises(capi.TpmError):
            ctx.set_fft_tiles(bad)


@pytest.mark.parametrize("prec", [P.PREC_FP64, P.PREC_MIXED])
def test_batch_matches_boxes_run_alone(capi, prec):
    """Boxes stepped together (one graph per step, a stream per box) are
    bit-identical to each box run alone; on the mixed path the 32-wide boxes
    take the TMA-fed passes."""
    shapes = [((16, 16, 16), 1000), ((24, 24, 24), 4000), ((32, 32, 32), 9000),
              ((32, 24, 16), 2500), ((16, 16, 16), 500)]
    cases = [case(dims=d, npart=n, seed=10 + i, heat=0.3 * (i % 2), prec=prec)
             for i, (d, n) in enumerate(shapes)]
    alone = [state(run(capi, p, s, 4)) for p, s in cases]
    for graph in (True, False):
        b = capi.Batch([p for p, _ in cases], [s.npart for _, s in cases])
        for box, (p, s) in zip(b.boxes, cases):
            box.load(s)
        b.autotune()
        for box in b.boxes:
            box.initialize()
        b.run(4, graph=graph)
        b.sync()
        for box, want in zip(b.boxes, alone):
            assert_same(state(box), want)
        b.close()

@pytest.mark.parametrize("prec,graph,npart", [(P.PREC_FP64, False, 6000),
                                              (P.PREC_MIXED, False, 6000),
                                              (P.PREC_MIXED, True, 6000), (P.PREC_MIXED, True, 0)])
def test_step_state_equals_load_step_save(capi, prec, graph, npart):
    """tpm_step_state (one call: load the host state, step, save it, the
    transfers overlapping the step) gives the bits of tpm_load_state +
    tpm_step + tpm_save_state, step after step, also in place and without
    particles; the context then steps on as usual."""
    import copy

    p, s = case(prec=prec, dims=(32, 32, 32), npart=npart, seed=21, heat=0.4)
    a = run(capi, p, s, 1)
    st0 = a.download_state()
    ref = copy.deepcopy(st0)
    b = capi.Context(p, s.npart)
    b.set_graph(graph)
    for _ in range(3):
        b.upload_state(ref)
        b.step()
        ref = b.download_state()
    c = capi.Context(p, s.npart)
    c.set_graph(graph)
    cur = copy.deepcopy(st0)
    for k in range(3):
        cur = c.step_state(cur, out=cur if k else None)
    for f in capi.Context.STATE_FIELDS:
        assert np.array_equal(cur[f], ref[f]), f
    if npart:
        for q in cur["part"]:
            assert np.array_equal(cur["part"][q], ref["part"][q]), q
        assert np.array_equal(cur["RHS_T"], ref["RHS_T"])
    else:
        assert cur["part"] is None and ref["part"] is None
    for k in ("P0", "T_cur", "num_timestep"):
        assert cur["scalars"][k] == ref["scalars"][k], k
    b.step()
    c.step()
    for f in ("RU", "RHO", "P", "C", "Q"):
        assert np.array_equal(b.download_field(f), c.download_field(f)), f
