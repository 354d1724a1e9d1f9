"""GB300-native Crank-Nicolson time step of GaDE (JVembe/dirac_hydrogen_code).

* :mod:`.gen`      — input generation in the reference file formats
                     (dumpCouplings + tools/main.py restatement)
* :mod:`.formats`  — readers/writers of the reference binary formats
* :mod:`.build`    — in-tree build of libgade_gb300.so and dirac_solver
* :mod:`.native`   — ctypes binding of the C ABI (include/gade.h)
* :mod:`.cn`       — the reference time loop driven from Python (one pulse,
                     or many pulses batched on one GPU)
* :mod:`.learned`  — learned initial guess (POD subspace + MLP) for
                     mixed-precision batches
"""
__all__ = ["gen", "formats", "build", "native", "cn", "learned"]
