"""CPU tests of the batched-pulse inputs: per-pulse radial tables against
the generator's files, the seeded pulse set, and batch creation errors
(status codes, no GPU compute)."""
import math

import numpy as np
import pytest

from dirac_hydrogen_code_gb300 import formats
from dirac_hydrogen_code_gb300.gen import generate
from dirac_hydrogen_code_gb300.gen.pulses import draw_pulses, pulse_tables


def test_pulse_tables_match_generated_files(workdirs, tmp_path):
    d, params, info = workdirs["tiny_nondipole"]
    omega, cycles = 37.5, 3
    d2 = str(tmp_path / "p")
    generate(dict(params, Omega=omega, Cycles=cycles), d2)
    g = pulse_tables(params, omega, cycles)
    assert g.shape == (6, info["lmax"], 4, info["blk_nnz"])
    for l in range(info["lmax"]):
        for a in range(6):
            for q in range(4):
                m = formats.csr_read(f"{d2}/g{q}a{a}l{l}.csr")
                scale = max(np.max(np.abs(m.Ax)), 1e-300)
                assert np.max(np.abs(m.Ax - g[a, l, q])) <= 1e-13 * scale
    # the problem's own Omega/Cycles reproduce its own files
    g0 = pulse_tables(params, params["Omega"], params["Cycles"])
    m = formats.csr_read(f"{d}/g2a4l1.csr")
    assert np.max(np.abs(m.Ax - g0[4, 1, 2])) <= 1e-13 * np.max(np.abs(m.Ax))


def test_draw_pulses_seeded():
    a, b = draw_pulses(64, 1234), draw_pulses(64, 1234)
    assert a == b and len(a) == 64
    assert a != draw_pulses(64, 1235)
    for p in a:
        assert 1.0 <= p["E0"] <= 100.0 and 10.0 <= p["omega"] <= 100.0
        assert p["cycles"] in (1, 2, 3) and p["ntime"] == 500 * p["cycles"]
        assert math.isclose(p["maxtime"], p["cycles"] * 2 * math.pi / p["omega"])
    assert {p["cycles"] for p in a} == {1, 2, 3}


def test_batch_create_errors_without_gpu(workdirs, native_lib):
    import torch
    from dirac_hydrogen_code_gb300.native import Batch, GadeError, Problem
    d, params, info = workdirs["tiny_dipole"]
    prob = Problem(d, info["lmax"])
    with pytest.raises(GadeError) as e:
        Batch(prob, [1e-3, 1e-3], chunk_splines=100)
    assert e.value.code == 4
    with pytest.raises(ValueError):
        Batch(prob, [1e-3, 1e-3], g=np.zeros((3, 6, info["lmax"], 4, info["blk_nnz"]), complex))
    if not torch.cuda.is_available():
        with pytest.raises(GadeError) as e:
            Batch(prob, [1e-3, 2e-3])
        assert e.value.code in (3, 4)
