"""flecsolve_gb300 -- GB300-native Krylov hot path of flecsolve.

The solvers, vector operations and CSR operator run as hand-written CUDA
kernels for sm_103a in ``libfsgpu.so`` behind the C ABI of
``include/fsgpu.h``; this package is the Python mirror of the reference's
API over that ABI (see :mod:`flecsolve_gb300.api`) plus the seeded problem
generators (:mod:`flecsolve_gb300.problems`).
"""
from . import build, problems  # noqa: F401


def __getattr__(name):
    # the CUDA-backed API is imported lazily so that the generators and the
    # build helpers work on hosts without a GPU
    if name in ("api", "batch_cg", "batch_tuning", "batch_schedule", "batch_format", "block_cg", "Context", "Vector", "Multi", "CSR", "SolveInfo", "op", "vec", "mat", "cg",
                "bicgstab", "gmres", "fcg", "pipelined_cg", "mixed_cg", "mixed_bicgstab", "mixed_gmres", "nka",
                "Shell"):
        import importlib
        api = importlib.import_module(__name__ + ".api")
        return api if name == "api" else getattr(api, name)
    raise AttributeError(name)
