"""GB300-native random-walk NMR walker path (CPMG and PFGSE walks) behind a C ABI.

Layers:
  * ``csrc/``       CUDA kernels for sm_103a and the C-ABI engine (include/rwnmr_gb300.h)
  * ``csrc/host``   C++ host frontend: config files, images, walker placement, sequences, CLI
  * ``engine``      ctypes binding of the engine
  * ``sim``         Python mirror of the reference's NMR_Simulation / NMR_cpmg / NMR_PFGSE API
  * ``autograd``    torch.autograd.Function wrappers (forward walk + seed-replay adjoint)
"""
from .engine import Batch, Engine, RwnmrError, fx_to_float, load_library, library_path  # noqa: F401

__all__ = ["Batch", "Engine", "RwnmrError", "fx_to_float", "load_library", "library_path"]
