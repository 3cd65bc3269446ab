"""Long runs compared on the statistics that characterise the flow: TKE,
dissipation rate, energy spectrum and particle radial distribution function,
within 2 %, GPU (FP64 and mixed) against the oracle over 100 RK4 steps of the
32^3 box with 10^4 particles (the CPU-runnable workload).
"""
import numpy as np
import pytest

from tpm import inputs, params as P

pytestmark = pytest.mark.gpu

TOL = 0.02
NSTEPS = 100


@pytest.fixture(scope="module")
def capi():
    from tpm import build, capi

    build.build()
    return capi


@pytest.fixture(scope="module")
def runs(capi, oracle_lib):
    w = P.WORKLOADS["box32_p1e4"]
    p = P.physical(w["N"], w["npart"], nu=w["nu"], A=w["A"], tau_p=w["tau_p"],
                   mass_loading=w["mass_loading"], heating_Q=w["heating_Q"])
    s = inputs.make_state(p, w["npart"], seed=w["seed"])
    p = p.replace(dt=inputs.cfl_dt(p, s.RU))
    o = oracle_lib.Oracle(p, s.npart)
    o.load(s)
    o.initialize()
    for _ in range(NSTEPS):
        o.step()
    ref = {"stats": o.statistics(), "RU": o.get_field("RU"), "RHO": o.get_field("RHO"),
           "part": o.get_particles(0)}
    out = {}
    for name, prec in (("fp64", P.PREC_FP64), ("mixed", P.PREC_MIXED)):
        ctx = capi.Context(p.replace(precision=prec), s.npart)
        ctx.load(s)
        ctx.initialize()
        ctx.set_graph(True)
        ctx.run(NSTEPS)
        ctx.sync()
        out[name] = ctx
    return p, ref, out


@pytest.mark.parametrize("name", ["fp64", "mixed"])
def test_tke_and_dissipation(runs, name):
    p, ref, out = runs
    st = out[name].statistics()
    for k in ("TKE", "dissipation", "u_rms", "C_var"):
        assert abs(st[k] - ref["stats"][k]) <= TOL * abs(ref["stats"][k]), (k, st[k], ref["stats"][k])


@pytest.mark.parametrize("name", ["fp64", "mixed"])
def test_energy_spectrum(runs, oracle_lib, name):
    p, ref, out = runs
    E, _ = out[name].spectrum()
    Er, _ = oracle_lib.spectrum(p, ref["RU"], ref["RHO"])
    sig = Er > 1e-3 * Er.max()  # the shells that carry the energy
    assert np.all(np.abs(E[sig] - Er[sig]) <= TOL * Er[sig])


@pytest.mark.parametrize("name", ["fp64", "mixed"])
def test_particle_rdf(runs, oracle_lib, name):
    p, ref, out = runs
    r_max, nb = 1.0, 10
    pairs, _ = out[name].rdf(r_max, nb)
    pr = ref["part"]
    want = oracle_lib.rdf_pairs(pr["x"], pr["y"], pr["z"], (p.Lx, p.Ly, p.Lz), r_max, nb)
    cum, cum_w = np.cumsum(pairs.astype(float)), np.cumsum(want.astype(float))
    assert np.all(np.abs(cum[2:] - cum_w[2:]) <= TOL * cum_w[2:])
