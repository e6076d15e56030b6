"""The Energybase adapter (include/faunus_gb300_energy.hpp) compiles against
the reference's own headers, as a maintainer would build it. CPU only; skipped
where the reference checkout is absent."""
import os
import subprocess

import pytest

from conftest import ROOT
from oracle.refdir import reference_dir

REF = reference_dir()


@pytest.mark.skipif(REF is None, reason="reference sources absent (set FG_REFERENCE_DIR)")
def test_adapter_compiles_against_reference_headers(tmp_path):
    cmd = ["g++", "-std=c++11", "-fsyntax-only", "-w",
           "-include", os.path.join(ROOT, "oracle", "ref", "compat.h"),
           "-I", os.path.join(REF, "include"), "-I", os.path.join(REF, "include", "eigen3"),
           "-I", os.path.join(ROOT, "include"), os.path.join(ROOT, "oracle", "ref", "adapter_check.cpp")]
    r = subprocess.run(cmd, capture_output=True, text=True, cwd=tmp_path)
    assert r.returncode == 0, r.stderr[-3000:]
