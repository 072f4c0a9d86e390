"""GB300-resident quantized H-matrix matvec (drop-in for qhmat's CUDA apply).

``HMatrix.load(path).matmul(x, device="cuda")`` replaces the reference's
``qhmat.HMatrix.matmul(x, device="cuda")``: the representation is uploaded
once and applied by hand-written sm_103a kernels through the C ABI declared in
``include/qhmat_gb300.h``.
"""

from ._lib import LIB_PATH, load_library
from .matrix import HMatrix, NativeHMatrix, PrecisionHMatrix, choose_form, precision_gate, qhmat_device_bytes

cuda_built = True

__all__ = ["HMatrix", "NativeHMatrix", "PrecisionHMatrix", "precision_gate", "choose_form", "LIB_PATH", "load_library",
           "cuda_built"]
