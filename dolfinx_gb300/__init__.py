"""dolfinx_gb300: DOLFINx's assembly + CG hot path on one GB300 (sm_103a).

Host set-up (mesh, dofmaps, sparsity) and every device kernel live in the
in-tree shared library ``_lib/libdfxgpu.so`` behind the C ABI of
``include/dfx_gpu.h``; this package is the Python mirror of the
reference's ``dolfinx.mesh`` / ``dolfinx.fem`` / ``dolfinx.la`` /
``dolfinx.graph`` / ``dolfinx.common`` calls, plus the matrix-free Q4
operator, the serving loop and the autotuner. Torch supplies device memory
and streams only.
"""

from . import _capi  # noqa: F401

__all__ = ["mesh", "fem", "la", "graph", "common", "log", "matrix_free", "serving", "autotune"]


def __getattr__(name):
    if name in __all__:
        import importlib

        return importlib.import_module(f"{__name__}.{name}")
    raise AttributeError(name)
