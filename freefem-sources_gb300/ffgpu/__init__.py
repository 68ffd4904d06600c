"""ffgpu: GB300-native assemble-and-solve for FreeFEM's varf/matrix/solve path.

See ``api`` for the FreeFEM-shaped interface and include/ffgpu.h for the C ABI.
"""
from .mesh import Mesh, square, cube, movemesh, jittered_square
from .fespace import FESpace
from .api import (BoundaryTerm, DeviceSpace, device_mesh, device_space, number_p2, number_p2_2d, Matrix, VarForm, context, fespace, kernel_launches, matrix, stream_handle,
                  matrix_from_csr, matrix_from_file, read_matrix_text, read_vector_text, rhs, varf_diffusion,
                  varf_elasticity, write_matrix_text, write_vector_text)
from ._lib import FFGPUError, lib

__all__ = ["Mesh", "square", "cube", "movemesh", "jittered_square", "FESpace", "DeviceSpace",
           "BoundaryTerm", "device_mesh", "device_space", "number_p2", "number_p2_2d", "Matrix", "VarForm", "context", "fespace", "kernel_launches", "matrix",
           "matrix_from_csr", "matrix_from_file", "read_matrix_text", "read_vector_text",
           "write_matrix_text", "write_vector_text", "rhs", "varf_diffusion", "varf_elasticity", "FFGPUError", "lib"]
