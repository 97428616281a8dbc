"""GB300 HSMM tensor-Viterbi: the reference's `tensor_viterbi.viterbi` entry
points for the CUDA backend."""
from .native import (  # noqa: F401
    Model,
    configure,
    decode_tensor_viterbi_cpp,
    decode_tensor_viterbi_cuda,
    decode_tensor_viterbi_cuda_loglik,
    decode_tensor_viterbi_omp,
)

__all__ = [
    "Model",
    "configure",
    "decode_tensor_viterbi_cpp",
    "decode_tensor_viterbi_cuda",
    "decode_tensor_viterbi_cuda_loglik",
    "decode_tensor_viterbi_omp",
]
