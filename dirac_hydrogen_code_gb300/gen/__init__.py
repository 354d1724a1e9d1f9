"""Input generation for the Crank-Nicolson step, in GaDE's file formats.

``generate(params, workdir)`` runs the dumpCouplings restatement followed by
the single-partition structure step, exactly as a user of the reference runs
``dumpCouplings input.json`` then ``python3 main.py``.
"""
from __future__ import annotations

from .couplings import dump_couplings, ik, imu, SOL  # noqa: F401
from .structure import build_structure  # noqa: F401

# Named workloads of the benchmark configurations (Z=1, rBox=30).
CONFIGS = {
    "dipole_small": dict(Nsplines=100, Ntime=500, Nkappa=4, Nmu=0, Nl=1, rBox=30.0,
                         Intensity=10, Omega=50.0, Cycles=1, Z=1),
    "nondipole_medium": dict(Nsplines=250, Ntime=1500, Nkappa=8, Nmu=4, Nl=0, rBox=30.0,
                             Intensity=10, Omega=50.0, Cycles=3, Z=1),
    "nondipole_large": dict(Nsplines=300, Ntime=4000, Nkappa=16, Nmu=8, Nl=10, rBox=30.0,
                            Intensity=10, Omega=50.0, Cycles=5, Z=1),
}


def generate(params: dict, workdir: str, verbose: bool = False) -> dict:
    info = dump_couplings(params, workdir, verbose=verbose)
    info.update(build_structure(workdir))
    return info
