"""Passive scalar transport on the GPU (grid::Update_Passive_Scalar,
grid.cpp:743-772): against the reference's own output (golden fixtures) and
the oracle, in FP64 (<= 1e-12 relative) and on the mixed path (<= 1e-5), and
through graph replay, restart files and statistics.
"""
import numpy as np
import pytest

from conftest import rel_err
from golden import SCALAR_NAMES, load
from tpm import inputs, params as P

pytestmark = pytest.mark.gpu

TOL = 1e-12
TOL_MIXED = 1e-5


@pytest.fixture(scope="module")
def capi():
    from tpm import build, capi

    build.build()
    return capi


def case(N=32, npart=5000, seed=41, s1_type=1, D_M=0.02, heat=0.5, prec=P.PREC_FP64):
    p = P.physical(N, npart, nu=0.02, A=0.1, tau_p=0.1, mass_loading=0.5, heating_Q=heat,
                   iterations=20, epsilon=1e-13, precision=prec)
    p = p.replace(solve_for_scalar=1, D_M=D_M, S1_type=s1_type)
    s = inputs.make_state(p, npart, seed=seed)
    s.PS = inputs.passive_scalar(p, seed)
    return p.replace(dt=inputs.cfl_dt(p, s.RU)), s


def run(capi, p, s, nsteps, graph=False):
    ctx = capi.Context(p, s.npart)
    ctx.load(s)
    ctx.initialize()
    if graph:
        ctx.set_graph(True)
    ctx.run(nsteps)
    ctx.sync()
    return ctx


@pytest.mark.parametrize("name", SCALAR_NAMES)
def test_scalar_matches_reference_golden(capi, name):
    p, s, ref, nsteps, _ = load(name)
    ctx = run(capi, p, s, nsteps)
    assert rel_err(ctx.download_field("PASSIVE_SCALAR"), ref["PS"]) <= TOL
    for f, k in (("RU", "RU"), ("RHO", "Rho"), ("P", "P")):
        assert rel_err(ctx.download_field(f), ref[k]) <= TOL, f


@pytest.mark.parametrize("s1_type", [0, 1])
def test_scalar_matches_oracle_ten_steps(capi, oracle_lib, s1_type):
    p, s = case(s1_type=s1_type)
    ctx = run(capi, p, s, 1)
    o = oracle_lib.Oracle(p, s.npart)
    o.load(s)
    o.initialize()
    o.step()
    assert rel_err(ctx.download_field("PASSIVE_SCALAR"), o.get_field("PASSIVE_SCALAR")) <= TOL
    ctx.run(9)
    for _ in range(9):
        o.step()
    assert rel_err(ctx.download_field("PASSIVE_SCALAR"), o.get_field("PASSIVE_SCALAR")) <= 1e-9
    st, so = ctx.statistics(), o.statistics()
    assert abs(st["Passive_Scalar_mean"] - so["Passive_Scalar_mean"]) <= 1e-9 * so["Passive_Scalar_mean"]


def test_scalar_mixed_and_graph(capi):
    p, s = case(s1_type=0, seed=42)
    f64 = run(capi, p, s, 3)
    graph = run(capi, p, s, 3, graph=True)
    assert np.array_equal(graph.download_field("PASSIVE_SCALAR"), f64.download_field("PASSIVE_SCALAR"))
    mixed = run(capi, p.replace(precision=P.PREC_MIXED), s, 3)
    assert rel_err(mixed.download_field("PASSIVE_SCALAR"), f64.download_field("PASSIVE_SCALAR")) <= TOL_MIXED


def test_scalar_restart_round_trip(capi, oracle_lib, tmp_path):
    p, s = case(N=24, npart=2000, seed=43)
    ctx = run(capi, p, s, 2)
    d = str(tmp_path)
    ctx.write_restart(d)
    r = inputs.read_restart(d, p)
    assert np.array_equal(r.PS, ctx.download_field("PASSIVE_SCALAR"))
    g = capi.Context(p, s.npart)
    g.read_restart(d)
    g.initialize()
    g.run(1)
    o = oracle_lib.Oracle(p, s.npart)
    o.load(r)
    o.initialize()
    o.step()
    assert rel_err(g.download_field("PASSIVE_SCALAR"), o.get_field("PASSIVE_SCALAR")) <= TOL
