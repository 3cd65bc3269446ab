"""Failure reporting through the C ABI: every fault is made on the host (bad
arguments, calls out of order, a non-finite value uploaded into the state) and
must come back as a status code with a message, never as a device trap, and
leave the context usable.
"""
import ctypes

import numpy as np
import pytest

from tpm import inputs, params as P

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def capi():
    from tpm import build, capi

    build.build()
    return capi


def case():
    p = P.physical(16, 500, nu=0.02, A=0.1, tau_p=0.1, mass_loading=0.3)
    s = inputs.make_state(p, 500, seed=12)
    return p.replace(dt=inputs.cfl_dt(p, s.RU)), s


def test_calls_out_of_order_and_bad_arguments(capi):
    p, s = case()
    ctx = capi.Context(p, s.npart)
    with pytest.raises(capi.TpmError) as e:
        ctx.step()  # before tpm_initialize
    assert e.value.code == -6
    ctx.load(s)
    ctx.initialize()
    with pytest.raises(capi.TpmError) as e:
        ctx.substep(4)
    assert e.value.code == -1
    L = capi.load_library()
    assert L.tpm_upload_field(ctx.h, 99, None) == -1
    assert L.tpm_download_field(ctx.h, 0, None) == -1
    with pytest.raises(capi.TpmError):
        ctx.rdf(-1.0, 10)
    # still usable
    ctx.step()
    ctx.sync()
    assert np.isfinite(ctx.download_field("RU")).all()


def test_non_finite_state_is_reported(capi):
    p, s = case()
    ctx = capi.Context(p, s.npart)
    ctx.load(s)
    RU = s.RU.copy()
    RU[0, 3, 4, 5] = np.nan
    ctx.upload_field("RU", RU)
    ctx.initialize()
    ctx.step()
    ctx.sync()
    with pytest.raises(capi.TpmError) as e:
        ctx.scalars()
    assert e.value.code == -4
    # a clean state uploaded afterwards steps normally
    ctx.load(s)
    ctx.initialize()
    ctx.step()
    assert np.isfinite(ctx.scalars()["P0"])
