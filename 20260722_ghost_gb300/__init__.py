"""GB300-native (sm_103a) body-of-revolution MoM monostatic RCS path.

Drop-in modules mirroring the reference project's entry points:

    bor_solver     solve_bor (PEC and surface impedance), solve_bor_dielectric
                   (PMCHWT), solve_bor_pec, solve_bor_batch, BorPecSolver, sphere_generatrix, ...
    batch          BorGpuBatch (size classes, CUDA-graph replay), Autotuner
    bor_streaming  StreamingFarBlocks, estimate_streaming_gb
    adjoint        bspline_rcs (torch.autograd.Function), ShapeGradient
    bor_dispatch   solve_monostatic_rcs_bor, solve_adaptive_frequency_sweep_bor,
                   bor_az_el_grid (.geo snapshots of conductors, impedance flags included)
    grim_io        export_result_to_grim, save_bor_az_el_grim
    materials      MaterialLibrary (the snapshot's impedance and medium tables)
    penetrable     DielectricBorProblem (the 4 Nn PMCHWT systems on the GPU)

All numerics run on one GPU through libghost_bor.so (C ABI in include/ghost_bor.h).
"""

from . import bodies, geometry  # noqa: F401
from .build import build  # noqa: F401

__all__ = ["bodies", "geometry", "build", "bor_solver", "bor_streaming", "engine", "batch", "adjoint",
           "bor_dispatch", "grim_io", "materials", "penetrable"]


def __getattr__(name):
    # the GPU modules import torch lazily so that a CPU-only import stays cheap
    if name in ("bor_solver", "bor_streaming", "engine", "batch", "_native", "adjoint", "bor_dispatch",
                "grim_io", "materials", "penetrable"):
        import importlib
        return importlib.import_module(f".{name}", __name__)
    raise AttributeError(name)
