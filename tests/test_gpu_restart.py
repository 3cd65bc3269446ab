"""Restart and dump files in the reference's byte formats.

tpm_write_restart writes the set that the reference's Initial=1 branch reads
(grid.cpp:221-238, particle.cpp:939-989); tpm_read_restart takes such a set
back; tpm_store writes the per-step dumps of grid::Store and
particle::Store_All (grid.cpp:525-592, particle.cpp:848-897).  The checks:
the files hold exactly the device state, a run continued from them on the GPU
matches the oracle continued from the same files, and a truncated set is
refused before anything is uploaded.
"""
import os

import numpy as np
import pytest

from conftest import rel_err
from tpm import inputs, params as P

pytestmark = pytest.mark.gpu

TOL = 1e-12  # FP64 parity bar of the one-step GPU tests


@pytest.fixture(scope="module")
def capi():
    from tpm import build, capi

    build.build()
    return capi


def case(seed=3):
    p = P.physical(32, 5_000, nu=0.02, A=0.1, tau_p=0.1, mass_loading=0.5, heating_Q=0.5,
                   iterations=20, epsilon=1e-13)
    s = inputs.make_state(p, 5_000, seed=seed)
    return p.replace(dt=inputs.cfl_dt(p, s.RU)), s


def test_write_restart_holds_device_state(capi, tmp_path):
    p, s = case()
    ctx = capi.Context(p, s.npart)
    ctx.load(s)
    ctx.initialize()
    ctx.run(2)
    ctx.sync()
    d = str(tmp_path)
    ctx.write_restart(d)
    r = inputs.read_restart(d, p)
    assert np.array_equal(r.RU, ctx.download_field("RU"))
    assert np.array_equal(r.Rho, ctx.download_field("RHO"))
    assert np.array_equal(r.P, ctx.download_field("P"))
    parts = ctx.download_particles("base")
    for q in inputs.PQ + ("flag",):
        assert np.array_equal(r.part[q], parts[q]), q
    sc = ctx.scalars()
    assert r.P0 == sc["P0"] and r.T_cur == sc["T_cur"]
    assert r.num_timestep == sc["num_timestep"] == 2


def test_restart_continues_like_oracle(capi, oracle_lib, tmp_path):
    p, s = case(seed=4)
    ctx = capi.Context(p, s.npart)
    ctx.load(s)
    ctx.initialize()
    ctx.run(3)
    ctx.sync()
    d = str(tmp_path)
    ctx.write_restart(d)
    ctx.close()

    g = capi.Context(p, s.npart)
    g.read_restart(d)
    g.initialize()
    g.run(2)
    g.sync()
    o = oracle_lib.Oracle(p, s.npart)
    o.load(inputs.read_restart(d, p))
    o.initialize()
    o.step()
    o.step()
    for f in ("RU", "RU_INT", "RHO", "P", "Q"):
        e = rel_err(g.download_field(f), o.get_field(f))
        assert e <= TOL, (f, e)
    a, b = g.download_particles("base"), o.get_particles(0)
    for q in inputs.PQ:
        assert rel_err(a[q], b[q]) <= TOL, q
    assert g.scalars()["num_timestep"] == 5


def test_store_dump_names_and_contents(capi, tmp_path):
    p, s = case(seed=5)
    ctx = capi.Context(p, s.npart)
    ctx.load(s)
    ctx.initialize()
    ctx.run(1)
    ctx.sync()
    d = str(tmp_path)
    ctx.store(d)
    shape = (p.Nz, p.Ny, p.Nx)
    rd = lambda n, dt=np.float64: np.fromfile(os.path.join(d, n), dtype=dt)
    assert np.array_equal(rd("RU_1.bin").reshape((3,) + shape), ctx.download_field("RU"))
    assert np.array_equal(rd("Rho_1.bin").reshape(shape), ctx.download_field("RHO"))
    assert np.array_equal(rd("P_1.bin").reshape(shape), ctx.download_field("P"))
    parts = ctx.download_particles("base")
    for q in inputs.PQ:
        assert np.array_equal(rd(f"Part_{q}_1.bin"), parts[q]), q
    assert np.array_equal(rd("Part_flag_1.bin", np.int32), parts["flag"])
    with open(os.path.join(d, "numbers_1.dat")) as f:
        tok = f.read().split()
    sc = ctx.scalars()
    assert float(tok[0]) == sc["P0"] and float(tok[1]) == sc["T_cur"] and int(tok[2]) == 1


def test_read_restart_refuses_truncated_set(capi, tmp_path):
    p, s = case(seed=6)
    d = str(tmp_path)
    inputs.write_restart(d, p, s)
    ctx = capi.Context(p, s.npart)
    with open(os.path.join(d, "Restart_Part_u.bin"), "r+b") as f:
        f.truncate(8 * (s.npart - 1))
    with pytest.raises(capi.TpmError):
        ctx.read_restart(d)
    with pytest.raises(capi.TpmError):
        ctx.read_restart(os.path.join(d, "missing"))
