"""CPU oracle of the SPH particle pipeline -- TEST INFRASTRUCTURE.

Only ``tests/``, ``__graft_entry__.smoke()`` and ``bench.py``'s cpu_baseline leg import
this package.  It is the checker: the product (``fluids_gb300``) never imports it.

``oracle.Oracle`` wraps ``sph_oracle.cpp`` (a C++ restatement of the reference kernels and
their host-side constant derivation, float or double, COMPAT or PHYSICS mode).
``oracle.refkernels`` wraps the reference's own OpenCL kernels compiled for the CPU through
``oracle/ref_shim`` (built by ``oracle/build_ref.sh`` where the reference is mounted);
those pin the oracle.
"""
from .oracle import (Oracle, OrcDerived, build_oracle, lib_path, STAGES, FIELDS,
                     WCSPH_STEP, morton3, stable_sort_pairs, kwargs_from_params)

__all__ = ["Oracle", "OrcDerived", "build_oracle", "lib_path", "STAGES", "FIELDS",
           "WCSPH_STEP", "morton3", "stable_sort_pairs", "kwargs_from_params"]
