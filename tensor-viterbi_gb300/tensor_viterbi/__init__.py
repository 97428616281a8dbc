"""GB300-native drop-in for the CUDA backend of the reference `tensor_viterbi`
package (tensor_viterbi/__init__.py there re-exports the same names)."""
from .viterbi.native import (  # noqa: F401
    Model,
    decode_tensor_viterbi_cpp,
    decode_tensor_viterbi_cuda,
    decode_tensor_viterbi_cuda_loglik,
    decode_tensor_viterbi_omp,
)

__all__ = [
    "Model",
    "decode_tensor_viterbi_cpp",
    "decode_tensor_viterbi_cuda",
    "decode_tensor_viterbi_cuda_loglik",
    "decode_tensor_viterbi_omp",
]
