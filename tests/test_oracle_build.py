"""The CPU oracle's recipe builds the C restatement on a host without the
reference's sources (as on the GPU hosts), and reports their absence through
its has-ref target instead of failing the default build."""
import os
import shutil
import subprocess

import pytest

from conftest import REPO


def test_oracle_builds_without_the_reference(tmp_path):
    if not shutil.which("make") or not shutil.which("gcc"):
        pytest.skip("make/gcc not available")
    shutil.copytree(os.path.join(REPO, "oracle"), tmp_path / "oracle",
                    ignore=shutil.ignore_patterns("_build", "_ref", "__pycache__"))
    shutil.copytree(os.path.join(REPO, "include"), tmp_path / "include")
    env = dict(os.environ, TPM_REFERENCE_DIR=str(tmp_path / "absent"))
    subprocess.check_call(["make", "-C", str(tmp_path / "oracle"), "-s"], env=env,
                          stdout=subprocess.DEVNULL)
    assert (tmp_path / "oracle" / "_build" / "liboracle.so").exists()
    r = subprocess.run(["make", "-C", str(tmp_path / "oracle"), "-s", "has-ref"], env=env,
                       capture_output=True)
    assert r.returncode != 0
