"""CPU-side checks of the C ABI boundary: libtpm.so loads and exports every
entry point include/tpm.h declares, the ctypes structs match the header, and
argument validation fails loudly without touching a GPU."""
import ctypes
import os
import re

import pytest

from conftest import REPO


@pytest.fixture(scope="module")
def lib():
    from tpm import build, capi

    build.build()
    return capi.load_library()


def declared_functions():
    text = open(os.path.join(REPO, "include", "tpm.h")).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(tpm_[a-z_0-9]+)\s*\(", text)))


def test_header_and_binding_agree():
    from tpm import capi

    assert set(declared_functions()) == set(capi.SIGNATURES)


def test_option_and_field_ids_match_the_header():
    """The harness's option and field ids are the header's enum values."""
    from tpm import capi

    text = re.sub(r"/\*.*?\*/", "", open(os.path.join(REPO, "include", "tpm.h")).read(), flags=re.S)
    opts = {m.group(1): int(m.group(2)) for m in re.finditer(r"\bTPM_OPT_([A-Z_0-9]+)\s*=\s*(\d+)", text)}
    assert opts and opts == {n[4:]: v for n, v in vars(capi).items() if n.startswith("OPT_")}
    body = re.search(r"TPM_FIELD_RU\s*=\s*0,(.*?)TPM_FIELD_COUNT", text, re.S).group(1)
    names = ["RU"] + re.findall(r"TPM_FIELD_([A-Z_0-9]+)", body)
    assert {n: i for i, n in enumerate(names)} == capi.FIELD


def test_library_exports_every_declared_symbol(lib):
    for name in declared_functions():
        assert hasattr(lib, name), name


def test_abi_version(lib):
    assert lib.tpm_abi_version() == 1


def test_params_struct_layout_matches_header():
    """sizeof/offsets of tpm_params as gcc lays out include/tpm.h."""
    import subprocess
    import tempfile

    from tpm.params import TpmParams, TpmScalars, TpmStats

    src = r'''
#include <stdio.h>
#include <stddef.h>
#include "tpm.h"
int main(void){
 printf("%zu %zu %zu %zu %zu %zu %zu %zu %zu\n", sizeof(tpm_params), offsetof(tpm_params, epsilon),
   offsetof(tpm_params, A1), offsetof(tpm_params, I02), sizeof(tpm_scalars),
   offsetof(tpm_scalars, max_abs_div), sizeof(tpm_stats), offsetof(tpm_stats, num_iteration),
   offsetof(tpm_stats, dissipation));
 return 0;}
'''
    with tempfile.TemporaryDirectory() as d:
        c = os.path.join(d, "t.c")
        open(c, "w").write(src)
        exe = os.path.join(d, "t")
        subprocess.check_call(["gcc", "-I", os.path.join(REPO, "include"), c, "-o", exe])
        got = list(map(int, subprocess.check_output([exe]).split()))
    want = [ctypes.sizeof(TpmParams), TpmParams.epsilon.offset, TpmParams.A1.offset,
            TpmParams.I02.offset, ctypes.sizeof(TpmScalars), TpmScalars.max_abs_div.offset,
            ctypes.sizeof(TpmStats), TpmStats.num_iteration.offset, TpmStats.dissipation.offset]
    assert got == want


def test_null_context_calls_fail_cleanly(lib):
    assert lib.tpm_step(None) == -1
    assert lib.tpm_destroy(None) == 0
    assert lib.tpm_launch_count(None) == 0
    assert lib.tpm_last_error(None) == b"null context"


def test_create_rejects_out_of_scope_options_before_touching_the_device(lib):
    from tpm.params import Params

    p = Params(Nx=16, Ny=16, Nz=16, solve_for_vector=1)
    h = ctypes.c_void_p()
    rc = lib.tpm_create(ctypes.byref(p.to_c()), 10, ctypes.byref(h))
    assert rc == -5  # TPM_ERR_UNSUPPORTED
    assert b"passive vector" in lib.tpm_last_error(h)
    lib.tpm_destroy(h)
    bad = Params(Nx=14, Ny=16, Nz=16)  # 14 = 2*7 does not factor into 2,3,5
    rc = lib.tpm_create(ctypes.byref(bad.to_c()), 10, ctypes.byref(h))
    assert rc == -1
    lib.tpm_destroy(h)


def test_null_context_state_and_option_calls_fail_cleanly(lib):
    """The host-state entry points and the options refuse a null context
    with TPM_ERR_ARG before touching any buffer or device."""
    n = None
    assert lib.tpm_step_state(n, n, n, n, n, n, n, 0.0, 0.0, 0, n, n, n, n, n, n, n) == -1
    assert lib.tpm_load_state(n, n, n, n, n, n, n, 0.0, 0.0, 0) == -1
    assert lib.tpm_save_state(n, n, n, n, n, n, n, n) == -1
    for opt in range(1, 6):
        assert lib.tpm_set_option(n, opt, 1) == -1
    assert lib.tpm_last_error(None) == b"null context"
