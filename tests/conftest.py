import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.join(ROOT, "oracle"))

# Small generated problems (seconds for the oracle) and the dipole benchmark
# configuration (Z=1, rBox=30, NSplines=100, NKappa=4, Nl=1, Omega=50, 1 cycle).
SMALL = {
    "tiny_dipole": dict(Nsplines=20, Ntime=40, Nkappa=2, Nmu=0, Nl=1, rBox=30.0,
                        Intensity=10, Omega=50.0, Cycles=1, Z=1),
    "tiny_nondipole": dict(Nsplines=24, Ntime=60, Nkappa=3, Nmu=2, Nl=0, rBox=30.0,
                           Intensity=10, Omega=50.0, Cycles=2, Z=1),
}


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300); runs through libgade_gb300")


@pytest.fixture(scope="session")
def workdirs(tmp_path_factory):
    from dirac_hydrogen_code_gb300.gen import CONFIGS, generate
    out = {}
    for name, params in list(SMALL.items()) + [("dipole_small", CONFIGS["dipole_small"])]:
        d = str(tmp_path_factory.mktemp(name))
        info = generate(params, d)
        out[name] = (d, params, info)
    return out


@pytest.fixture(scope="session")
def native_lib():
    from dirac_hydrogen_code_gb300 import build, native
    if build.is_stale():
        build.build()
    return native.load_library()
