"""GB300-native random-walk NMR walker path (CPMG and PFGSE walks) behind a C ABI.

Layers:
  * ``csrc/``       CUDA kernels for sm_103a and the C-ABI engine (include/rwnmr_gb300.h)
  * ``csrc/host``   C++ host frontend: config files, images, walker placement, sequences, CLI
  * ``engine``      ctypes binding of the engine (single-image contexts, batches, device allocator)
  * ``host``        ctypes binding of the host frontend (images, placement, configs, T2 inversion)
  * ``autograd``    torch.autograd.Function wrappers (forward walk with its sensitivities, or the
                    seed-replay adjoint)
  * ``fit``, ``ga`` relaxivity fits on the GPU walk and the restated genetic-algorithm baseline
  * ``shard``       walker sharding over ranks with one exact integer all-reduce
"""
from .engine import (Batch, Engine, RwnmrError, fx_to_float, library_path, load_library,  # noqa: F401
                     set_device_allocator, use_torch_allocator)

__all__ = ["Batch", "Engine", "RwnmrError", "fx_to_float", "load_library", "library_path",
           "set_device_allocator", "use_torch_allocator"]
